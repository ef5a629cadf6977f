"""Adjoint of the raw periodic-box bispectrum: gradients against central
finite differences of the FP64 forward estimate, FP32-mixed against FP64,
and the autograd wrapper against the direct adjoint."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from triumvirate_gb300.adjoint import (BispecGppConfig,  # noqa: E402
                                       _forward, bispec_gpp,
                                       bispec_gpp_adjoint)
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
    b = bispec_gpp(pos, w, cfg)
    lam = torch.linspace(-1., 1., b.numel(), dtype=torch.float64,
                         device=b.device)
    (b * lam).sum().backward()
    g = bispec_gpp_adjoint(pos.detach(), w.detach(), lam.cpu().numpy(), cfg)
    for got, ref in ((w.grad, g['grad_w']), (pos.grad, g['grad_pos'])):
        assert torch.max(torch.abs(got - ref)) <= \
            1e-5 * torch.max(torch.abs(ref))
