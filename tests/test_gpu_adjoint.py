"""Adjoint of the periodic-box bispectrum (raw and shot noise): gradients
against central finite differences of the FP64 forward estimate,
FP32-mixed against FP64, the autograd wrappers against the direct
adjoint, and the chi^2 gradient of a 256^3, 5e5-particle TSC estimate
with respect to positions, weights and a count mesh."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from triumvirate_gb300.adjoint import (BispecGppConfig,  # noqa: E402
                                       _forward, bispec_gpp,
                                       bispec_gpp_adjoint, bispec_gpp_mesh,
                                       bispec_gpp_vjp)
from triumvirate_gb300.dataobjs import Binning  # noqa: E402

BOX, NGRID, N = 600., 32, 4000


def _inputs(seed=5, n=N):
    rng = np.random.default_rng(seed)
    pos = torch.from_numpy(rng.uniform(0., BOX, (n, 3))).cuda()
    w = torch.from_numpy(rng.uniform(0.5, 1.5, n)).cuda()
    return pos, w


def _cfg(precision='fp64', form='diag', assignment='tsc'):
    return BispecGppConfig(BOX, NGRID, Binning('fourier', 'lin', 0.02, 0.12, 5),
                           assignment=assignment, form=form,
                           precision=precision)


def _loss(pos, w, cfg, lam):
    return float(np.dot(lam, _forward(pos, w, cfg)['bk_raw'].real))


@pytest.mark.parametrize("assignment", ['cic', 'tsc', 'pcs'])
def test_weight_gradient_matches_finite_differences(assignment):
    cfg = _cfg(assignment=assignment)
    pos, w = _inputs()
    lam = np.random.default_rng(1).normal(size=cfg.dim)
    g = bispec_gpp_adjoint(pos, w, lam, cfg)
    gw = g['grad_w'].cpu().numpy()
    h = 1e-3
    for i in (0, 17, 1234, N - 1):
        wp, wm = w.clone(), w.clone()
        wp[i] += h
        wm[i] -= h
        fd = (_loss(pos, wp, cfg, lam) - _loss(pos, wm, cfg, lam)) / (2 * h)
        assert abs(fd - gw[i]) <= 1e-6 * np.max(np.abs(gw)), (i, fd, gw[i])


def test_position_gradient_matches_finite_differences():
    cfg = _cfg()
    pos, w = _inputs()
    lam = np.random.default_rng(2).normal(size=cfg.dim)
    g = bispec_gpp_adjoint(pos, w, lam, cfg)
    gp = g['grad_pos'].cpu().numpy()
    h = 1e-2    # Mpc/h
    scale = np.max(np.abs(gp))
    for i in (3, 222, 3001):
        for a in range(3):
            pp, pm = pos.clone(), pos.clone()
            pp[i, a] += h
            pm[i, a] -= h
            fd = (_loss(pp, w, cfg, lam) - _loss(pm, w, cfg, lam)) / (2 * h)
            assert abs(fd - gp[i, a]) <= 1e-4 * scale, (i, a, fd, gp[i, a])


def test_forward_values_and_full_form():
    cfg = _cfg(form='full')
    pos, w = _inputs(7)
    lam = np.random.default_rng(3).normal(size=cfg.dim)
    g = bispec_gpp_adjoint(pos, w, lam, cfg)
    ref = _forward(pos, w, cfg)['bk_raw']
    assert np.max(np.abs(g['raw'] - ref)) <= 1e-10 * np.max(np.abs(ref))
    gw = g['grad_w'].cpu().numpy()
    h = 1e-3
    for i in (9, 2500):
        wp, wm = w.clone(), w.clone()
        wp[i] += h
        wm[i] -= h
        fd = (_loss(pos, wp, cfg, lam) - _loss(pos, wm, cfg, lam)) / (2 * h)
        assert abs(fd - gw[i]) <= 1e-6 * np.max(np.abs(gw))


def test_fp32mixed_gradient_matches_fp64():
    pos, w = _inputs(11)
    lam = np.random.default_rng(4).normal(size=_cfg().dim)
    g64 = bispec_gpp_adjoint(pos, w, lam, _cfg('fp64'), mesh=True)
    g32 = bispec_gpp_adjoint(pos, w, lam, _cfg('fp32mixed'), mesh=True)
    for k in ('grad_w', 'grad_pos', 'grad_mesh'):
        a, b = g32[k].cpu().numpy(), g64[k].cpu().numpy()
        assert np.max(np.abs(a - b)) <= 1e-4 * np.max(np.abs(b)), k


def test_mesh_gradient_gathers_to_weight_gradient():
    """dL/dw_i is the mesh gradient interpolated with the window; for NGP
    that is the gradient of the particle's own cell."""
    cfg = _cfg(assignment='ngp')
    pos, w = _inputs(12)
    lam = np.random.default_rng(6).normal(size=cfg.dim)
    g = bispec_gpp_adjoint(pos, w, lam, cfg, mesh=True)
    gm = g['grad_mesh'].cpu().numpy()
    p = pos.cpu().numpy()
    loc = NGRID * p / BOX
    idx = np.floor(loc).astype(int)
    idx = np.where(loc - idx >= 0.5, (idx + 1) % NGRID, idx)
    expect = gm[idx[:, 0], idx[:, 1], idx[:, 2]]
    assert np.allclose(g['grad_w'].cpu().numpy(), expect, rtol=1e-12,
                       atol=1e-12 * np.max(np.abs(expect)))


def test_autograd_matches_direct_adjoint():
    cfg = _cfg('fp32mixed')
    pos, w = _inputs(13)
    pos.requires_grad_(True)
    w.requires_grad_(True)
    b = bispec_gpp(pos, w, cfg, shot_noise=False)
    lam = torch.linspace(-1., 1., b.numel(), dtype=torch.float64,
                         device=b.device)
    (b * lam).sum().backward()
    g = bispec_gpp_adjoint(pos.detach(), w.detach(), lam.cpu().numpy(), cfg)
    for got, ref in ((w.grad, g['grad_w']), (pos.grad, g['grad_pos'])):
        assert torch.max(torch.abs(got - ref)) <= \
            1e-5 * torch.max(torch.abs(ref))


def _loss_b(pos, w, cfg, lam):
    """lam . Re(raw - shot) of the forward estimate."""
    r = _forward(pos, w, cfg)
    return float(np.dot(lam, (r['bk_raw'] - r['bk_shot']).real))


@pytest.mark.parametrize("form", ['diag', 'full'])
def test_shot_noise_gradient_matches_finite_differences(form):
    """The shot noise's single-leg (two-point statistics) and pair (xi)
    terms differentiated with the raw part."""
    cfg = _cfg(form=form)
    pos, w = _inputs(21)
    lam = np.random.default_rng(8).normal(size=cfg.dim)
    g = bispec_gpp_vjp(cfg, lam, -lam, positions=pos, weights=w)
    gw, gp = g['grad_w'].cpu().numpy(), g['grad_pos'].cpu().numpy()
    for i in (5, 1777, N - 2):
        wp, wm = w.clone(), w.clone()
        wp[i] += 1e-3
        wm[i] -= 1e-3
        fd = (_loss_b(pos, wp, cfg, lam) - _loss_b(pos, wm, cfg, lam)) / 2e-3
        assert abs(fd - gw[i]) <= 1e-6 * np.max(np.abs(gw)), (i, fd, gw[i])
        for a in range(3):
            pp, pm = pos.clone(), pos.clone()
            pp[i, a] += 1e-2
            pm[i, a] -= 1e-2
            fd = (_loss_b(pp, w, cfg, lam) - _loss_b(pm, w, cfg, lam)) / 2e-2
            assert abs(fd - gp[i, a]) <= 1e-4 * np.max(np.abs(gp)), \
                (i, a, fd, gp[i, a])


def test_autograd_without_weights_matches_vjp():
    """Unit weights: no weight column, no weight gradient."""
    cfg = _cfg('fp32mixed')
    pos, _ = _inputs(14)
    pos.requires_grad_(True)
    b = bispec_gpp(pos, None, cfg)
    lam = torch.linspace(-1., 1., b.numel(), dtype=torch.float64,
                         device=b.device)
    (b * lam).sum().backward()
    g = bispec_gpp_vjp(cfg, lam.cpu().numpy(), -lam.cpu().numpy(),
                       positions=pos.detach(), weights=None)
    assert torch.max(torch.abs(pos.grad - g['grad_pos'])) <= \
        1e-5 * torch.max(torch.abs(g['grad_pos']))


def test_mesh_function_gradient_matches_finite_differences():
    """Raw B_000 of a count mesh: the autograd function's gradient against
    central differences of single cells (FP64 path)."""
    cfg = _cfg()
    cfg.norm = 1e-3
    gen = torch.Generator(device='cuda').manual_seed(3)
    m = (torch.rand((NGRID,) * 3, generator=gen, device='cuda') *
         0.25).to(torch.float32)
    m.requires_grad_(True)
    lam = torch.from_numpy(np.random.default_rng(9).normal(
        size=cfg.dim)).cuda()
    (bispec_gpp_mesh(m, cfg) * lam).sum().backward()
    gm = m.grad.double().cpu().numpy()
    assert abs(gm.mean()) <= 1e-9 * np.max(np.abs(gm))

    def loss(mm):
        return float((bispec_gpp_mesh(mm, cfg) * lam).sum())
    h = 2. ** -12
    for c in ((0, 0, 0), (3, 17, 30), (31, 8, 5)):
        mp, mm = m.detach().clone(), m.detach().clone()
        mp[c] += h
        mm[c] -= h
        fd = (loss(mp) - loss(mm)) / (2 * h)
        assert abs(fd - gm[c]) <= 1e-6 * np.max(np.abs(gm)), (c, fd, gm[c])


# ---------------------------------------------------------------------------
# chi^2 = sum_b (B_b - T_b)^2 / sigma_b^2 of B_000 = raw - shot on 16
# diagonal bins 0.01-0.16 h/Mpc, 256^3 mesh, 5e5 TSC particles; T_b and
# sigma_b from a seeded FP64 estimate of another catalogue.
# ---------------------------------------------------------------------------

BOX4, NG4, N4 = 1000., 256, 500_000


@pytest.fixture(scope='module')
def chi2_case():
    bins = Binning('fourier', 'lin', 0.01, 0.16, 16)
    cfg64 = BispecGppConfig(BOX4, NG4, bins, assignment='tsc',
                            precision='fp64')
    cfg32 = BispecGppConfig(BOX4, NG4, bins, assignment='tsc',
                            precision='fp32mixed')
    rng = np.random.default_rng(40)
    pos = torch.from_numpy(rng.uniform(0., BOX4, (N4, 3))).cuda()
    w = torch.from_numpy(rng.uniform(0.8, 1.2, N4)).cuda()
    pos_t = torch.from_numpy(np.random.default_rng(41).uniform(
        0., BOX4, (N4, 3))).cuda()
    rt = _forward(pos_t, None, cfg64)
    T = (rt['bk_raw'] - rt['bk_shot']).real
    sigma = 0.05 * np.abs(T) + 1e-3 * np.max(np.abs(T))
    return cfg64, cfg32, pos, w, T, sigma


def _chi2_and_cotangent(cfg, pos, w, T, sigma):
    r = _forward(pos, w, cfg)
    B = (r['bk_raw'] - r['bk_shot']).real
    return float(np.sum((B - T) ** 2 / sigma ** 2)), 2. * (B - T) / sigma ** 2


def _away_from_breakpoints(p, h):
    """TSC windows change form where the cell offset is 0 or 1/2: central
    differences across such a point lose their second order."""
    s = (p * NG4 / BOX4) % 1.
    d = np.minimum.reduce([s, np.abs(s - 0.5), 1. - s])
    return np.all(d > 4 * h * NG4 / BOX4)


def test_chi2_gradients_at_adjoint_config(chi2_case):
    cfg64, cfg32, pos, w, T, sigma = chi2_case
    _, lam = _chi2_and_cotangent(cfg64, pos, w, T, sigma)
    g64 = bispec_gpp_vjp(cfg64, lam, -lam, positions=pos, weights=w)
    _, lam32 = _chi2_and_cotangent(cfg32, pos, w, T, sigma)
    g32 = bispec_gpp_vjp(cfg32, lam32, -lam32, positions=pos, weights=w)
    gw64, gp64 = g64['grad_w'].cpu().numpy(), g64['grad_pos'].cpu().numpy()
    gw32, gp32 = g32['grad_w'].cpu().numpy(), g32['grad_pos'].cpu().numpy()
    # FP32-mixed against the FP64 adjoint.
    assert np.max(np.abs(gw32 - gw64)) <= 1e-4 * np.max(np.abs(gw64))
    assert np.max(np.abs(gp32 - gp64)) <= 1e-4 * np.max(np.abs(gp64))
    # Central differences of the FP64 chi^2 (steps 1e-3 in weight, 1e-2
    # Mpc/h in position) on sampled particles.
    p_host = pos.cpu().numpy()
    hp, hw = 1e-2, 1e-3
    picks = [i for i in np.random.default_rng(42).choice(N4, 60, False)
             if _away_from_breakpoints(p_host[i], hp)][:5]
    assert len(picks) >= 3

    def chi2(pp, ww):
        return _chi2_and_cotangent(cfg64, pp, ww, T, sigma)[0]
    for i in picks:
        wp, wm = w.clone(), w.clone()
        wp[i] += hw
        wm[i] -= hw
        fd = (chi2(pos, wp) - chi2(pos, wm)) / (2 * hw)
        for g in (gw64, gw32):
            assert abs(fd - g[i]) <= 1e-4 * abs(fd) + \
                1e-6 * np.max(np.abs(gw64)), (i, fd, g[i])
        for a in range(3):
            pp, pm = pos.clone(), pos.clone()
            pp[i, a] += hp
            pm[i, a] -= hp
            fd = (chi2(pp, w) - chi2(pm, w)) / (2 * hp)
            for g in (gp64, gp32):
                assert abs(fd - g[i, a]) <= 1e-4 * abs(fd) + \
                    1e-6 * np.max(np.abs(gp64)), (i, a, fd, g[i, a])


def test_chi2_mesh_gradient_at_adjoint_config(chi2_case):
    """chi^2 of raw B_000 of the 256^3 count mesh (FP32 tensor input)."""
    cfg64, cfg32, pos, w, T, sigma = chi2_case
    from triumvirate_gb300 import _engine
    pc = _engine.make_params(
        {'boxsize': {a: BOX4 for a in 'xyz'},
         'ngrid': {a: NG4 for a in 'xyz'}, 'assignment_order': 3,
         'interlace': False, 'degrees': {}, 'form': 'diag',
         'precision': 'fp64', 'verbose': 0}, '2pt')
    cols = [pos[:, a].contiguous() for a in range(3)]
    torch.cuda.synchronize()
    cat = _engine.device_catalogue(N4, *(c.data_ptr() for c in cols))
    # The count mesh: the weighted density times the cell volume.
    vcell = (BOX4 / NG4) ** 3
    mesh = torch.from_numpy(_engine.assign_mesh(cfg64.ctx, pc, cat) *
                            vcell).to(torch.float32).cuda()
    del cols
    for cfg in (cfg64, cfg32):
        cfg.norm = cfg64.norm_for(N4)
    Tm = T * 1.1
    sig = 0.05 * np.abs(Tm) + 1e-3 * np.max(np.abs(Tm))

    def chi2(m, cfg):
        b = bispec_gpp_mesh(m, cfg)
        tt = torch.from_numpy(Tm).cuda()
        ss = torch.from_numpy(sig).cuda()
        return (((b - tt) / ss) ** 2).sum()
    try:
        grads = []
        for cfg in (cfg64, cfg32):
            m = mesh.clone().requires_grad_(True)
            chi2(m, cfg).backward()
            grads.append(m.grad.double().cpu().numpy())
        g64, g32 = grads
        assert np.max(np.abs(g32 - g64)) <= 1e-4 * np.max(np.abs(g64))
        h = 2. ** -10
        for c in ((0, 0, 0), (100, 31, 7), (255, 128, 64), (17, 200, 99)):
            mp, mm = mesh.clone(), mesh.clone()
            mp[c] += h
            mm[c] -= h
            fd = (float(chi2(mp, cfg64)) - float(chi2(mm, cfg64))) / (2 * h)
            assert abs(fd - g64[c]) <= 1e-4 * abs(fd) + \
                1e-6 * np.max(np.abs(g64)), (c, fd, g64[c])
    finally:
        for cfg in (cfg64, cfg32):
            cfg.norm = None
