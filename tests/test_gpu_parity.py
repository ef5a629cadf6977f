"""GPU parity: the CUDA path (through the C ABI) against the reference's
golden files and against the CPU oracle on seeded inputs.

Tolerances: FP64 path -- the reference tests' own ``np.allclose`` (rtol
1e-5, atol 1e-8; shot noise atol 1e-6) against the goldens, and 1e-9
relative to each entry's complex modulus against the oracle.  FP32-mixed
path -- 1e-5 relative to each entry's complex modulus against the oracle
or the FP64 path (``assert_per_bin``), and the reference tests' own
``np.allclose`` against the goldens.  Two FP32-mixed runs (whose FP32
atomics deposit in different orders) agree per entry to twice that.
Mode / pair counts must be identical in both.
"""
import numpy as np
import pytest

from conftest import BOX, KBINS, NMESH, RBINS, THREEPT_CASES, load_golden
from oracle import trv_oracle as O
from test_oracle import (WINDOW_CASES, _window_rand, check_powspec,
                         check_threept)
from triumvirate_gb300 import _engine, _lib
from triumvirate_gb300.catalogue import ParticleCatalogue
from triumvirate_gb300.dataobjs import Binning
from triumvirate_gb300.threept import (compute_3pcf, compute_3pcf_in_gpp_box,
                                       compute_3pcf_window, compute_bispec,
                                       compute_bispec_in_gpp_box)
from triumvirate_gb300.twopt import (compute_powspec,
                                     compute_powspec_in_gpp_box)

pytestmark = pytest.mark.gpu

PRECISIONS = ['fp64', 'fp32mixed']


def _sampling(precision, ngrid=NMESH, assignment='tsc', interlace=False,
              box=BOX):
    return {'boxsize': [box] * 3 if np.isscalar(box) else list(box),
            'ngrid': [ngrid] * 3 if np.isscalar(ngrid) else list(ngrid),
            'assignment': assignment, 'interlace': interlace,
            'precision': precision}


def _cats(d, r=None):
    dc = ParticleCatalogue(d[:, 0], d[:, 1], d[:, 2], nz=d[:, 3])
    if r is None:
        return dc
    return dc, ParticleCatalogue(r[:, 0], r[:, 1], r[:, 2], nz=r[:, 3])


def rel_err(a, b):
    a, b = np.asarray(a), np.asarray(b)
    scale = np.maximum(np.abs(b), 1e-300)
    return float(np.max(np.abs(a - b) / scale))


# Per-entry relative bound of the FP32-mixed path against FP64 / the oracle:
# bispectra whose shell fields take the float-float transforms (real
# periodic-box fields: every leg of order m = 0 and even degree), and the
# other FP32-mixed paths, whose transforms are plain FP32 FFTs (complex or
# odd-degree legs, survey fields, the 3PCF's j_l-weighted fields, and the
# FP64-field options that start from the FP32 mesh spectrum).
RTOL_FP32 = 1e-5
RTOL_FP32_FFT = 2e-4


def fp32_rtol(kind, degrees, survey=False):
    """Per-entry bound of an FP32-mixed estimate of this kind."""
    ell1, ell2 = degrees[0], degrees[1]
    if kind == 'bispec' and not survey and ell1 % 2 == 0 and ell2 == 0:
        return RTOL_FP32
    return RTOL_FP32_FFT


def assert_close_threept(res, ref, kind, precision, rtol=RTOL_FP32):
    keys = (['k1_bin', 'k1_eff', 'nmodes_1', 'k2_bin', 'k2_eff', 'nmodes_2',
             'bk_raw', 'bk_shot'] if kind == 'bispec' else
            ['r1_bin', 'r1_eff', 'npairs_1', 'r2_bin', 'r2_eff', 'npairs_2',
             'zeta_raw', 'zeta_shot'])
    assert np.array_equal(res[keys[2]], ref[keys[2]])
    assert np.array_equal(res[keys[5]], ref[keys[5]])
    assert np.allclose(res[keys[0]], ref[keys[0]], rtol=1e-15, atol=0)
    assert np.allclose(res[keys[1]], ref[keys[1]], rtol=1e-12, atol=0)
    for k in keys[6:]:
        assert_close_vector(res[k], ref[k], precision, k, rtol)


def assert_per_bin(got, ref, label='', rtol=RTOL_FP32):
    """|got - ref| <= rtol |ref| for every entry (complex modulus).  Entries
    that are zero by symmetry (|ref| below 1e-13 of the largest) must be
    zero to that level."""
    got, ref = np.asarray(got), np.asarray(ref)
    err = np.abs(got - ref)
    mod = np.abs(ref)
    scale = float(np.max(mod)) if mod.size else 0.
    bound = rtol * mod + 1e-13 * scale
    rel = err / np.maximum(mod, 1e-300)
    worst = int(np.argmax(np.where(mod > 1e-13 * scale, rel, 0.))) \
        if mod.size else 0
    assert np.all(err <= bound), '%s: max per-bin rel err %.3g at %d, |ref|/max %.3g' % (
        label, float(rel.flat[worst]), worst,
        float(mod.flat[worst] / scale) if scale else 0.)


def assert_close_vector(got, ref, precision, label='', rtol=RTOL_FP32):
    if precision == 'fp64':
        err = np.abs(np.asarray(got) - np.asarray(ref))
        scale = float(np.max(np.abs(ref)))
        bound = 1e-9 * np.abs(ref) + 1e-12 * scale
        assert np.all(err <= bound), (label, float(np.max(err) / scale))
    else:
        assert_per_bin(got, ref, label, rtol)


# ---------------------------------------------------------------------------
# Golden files (reference tests/test_threept.py, tests/test_twopt.py)
# ---------------------------------------------------------------------------

@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("kind, degrees, form, idx_bin, golden",
                         THREEPT_CASES)
def test_golden_gpp(precision, kind, degrees, form, idx_bin, golden,
                    data_catalogue_array):
    cat = _cats(data_catalogue_array)
    bins = (Binning('fourier', 'lin', *KBINS) if kind == 'bispec'
            else Binning('config', 'lin', *RBINS))
    fn = compute_bispec_in_gpp_box if kind == 'bispec' \
        else compute_3pcf_in_gpp_box
    res = fn(cat, degrees=degrees, binning=bins, form=form, idx_bin=idx_bin,
             sampling_params=_sampling(precision))
    _check_golden(res, load_golden(golden.format('gpp')), kind, precision,
                  degrees)


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("kind, degrees, form, idx_bin, golden",
                         THREEPT_CASES)
def test_golden_lpp(precision, kind, degrees, form, idx_bin, golden,
                    data_catalogue_array, rand_catalogue_array):
    dc, rc = _cats(data_catalogue_array, rand_catalogue_array)
    bins = (Binning('fourier', 'lin', *KBINS) if kind == 'bispec'
            else Binning('config', 'lin', *RBINS))
    fn = compute_bispec if kind == 'bispec' else compute_3pcf
    res = fn(dc, rc, degrees=degrees, binning=bins, form=form,
             idx_bin=idx_bin, sampling_params=_sampling(precision))
    _check_golden(res, load_golden(golden.format('lpp')), kind, precision,
                  degrees, survey=True)


def _check_golden(res, ext, kind, precision, degrees=(0, 0, 0),
                  survey=False):
    """FP64 and the float-float FP32-mixed bispectra: the reference test
    verbatim (``np.allclose``, rtol 1e-5 per entry, atol 1e-8 and 1e-6 on
    shot noise); the FP32-FFT paths the same with rtol 2e-4."""
    rtol = 1e-5 if precision == 'fp64' else fp32_rtol(kind, degrees, survey)
    check_threept(res, ext, kind, rtol=rtol)


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("degrees, form, idx_bin, golden", WINDOW_CASES)
def test_golden_3pcf_window(precision, degrees, form, idx_bin, golden,
                            rand_catalogue_array):
    """Reference tests/test_threept.py:265-332 (3PCF window)."""
    r = rand_catalogue_array
    rc = ParticleCatalogue(r[:, 0], r[:, 1], r[:, 2], nz=r[:, 3])
    res = compute_3pcf_window(rc, degrees=degrees,
                              binning=Binning('config', 'lin', *RBINS),
                              form=form, idx_bin=idx_bin,
                              sampling_params=_sampling(precision))
    _check_golden(res, load_golden(golden), '3pcf', precision, degrees,
                  survey=True)


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("degrees, wa", [((0, 0, 0), (1, 1)),
                                         ((2, 0, 2), (0, 1))])
def test_3pcf_window_wide_angle_matches_oracle(precision, degrees, wa,
                                               rand_catalogue_array):
    """The wide-angle kernel r^-(i_wa + j_wa) on G (field.cpp:1727-1760)
    has no golden file; the oracle is the reference."""
    r = rand_catalogue_array
    rc = ParticleCatalogue(r[:, 0], r[:, 1], r[:, 2], nz=r[:, 3])
    res = compute_3pcf_window(rc, degrees=degrees, wa_orders=wa,
                              binning=Binning('config', 'lin', *RBINS),
                              form='diag', sampling_params=_sampling(precision))
    p = O.Params(BOX, NMESH, 'tsc', False, *degrees, form='diag')
    edges, centres = O.lin_binning(*RBINS)
    norm = O.bispec_norm_from_particles(r[:, 3], 1., 1.)
    ref = O.compute_3pcf_window(_window_rand(r), p, edges, centres, norm,
                                wide_angle=True, i_wa=wa[0], j_wa=wa[1])
    assert_close_threept(res, ref, '3pcf', precision,
                         fp32_rtol('3pcf', degrees, survey=True))


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("ell", [0, 2])
def test_golden_powspec(precision, ell, data_catalogue_array,
                        rand_catalogue_array):
    bins = Binning('fourier', 'lin', *KBINS)
    res = compute_powspec_in_gpp_box(_cats(data_catalogue_array), degree=ell,
                                     binning=bins,
                                     sampling_params=_sampling(precision))
    check_powspec(res, load_golden(f"pk{ell}_gpp.txt"))
    dc, rc = _cats(data_catalogue_array, rand_catalogue_array)
    res = compute_powspec(dc, rc, degree=ell, binning=bins,
                          sampling_params=_sampling(precision))
    check_powspec(res, load_golden(f"pk{ell}_lpp.txt"))


# ---------------------------------------------------------------------------
# Seeded catalogues against the oracle
# ---------------------------------------------------------------------------

def _uniform(n, box, seed):
    rng = np.random.default_rng(seed)
    return rng.uniform(0., box, size=(n, 3))


def _oracle_gpp(kind, pos, box, ngrid, assignment, degrees, form, idx_bin,
                bins):
    x, y, z = O.periodise(pos[:, 0], pos[:, 1], pos[:, 2], [box] * 3)
    p = O.Params(box, ngrid, assignment, False, *degrees, form=form,
                 idx_bin=idx_bin)
    edges, centres = O.lin_binning(*bins)
    n = pos.shape[0]
    norm = O.bispec_norm_from_particles(np.full(n, n / box ** 3), 1., 1.)
    fn = (O.compute_bispec_in_gpp_box if kind == 'bispec'
          else O.compute_3pcf_in_gpp_box)
    return fn(np.stack([x, y, z], -1), p, edges, centres, norm)


GPP_CASES = [
    # kind, assignment, ngrid, degrees, form, idx_bin, bins
    ('bispec', 'tsc', 32, (0, 0, 0), 'diag', None, (0.01, 0.1, 5)),
    ('bispec', 'ngp', 32, (0, 0, 0), 'full', None, (0.01, 0.1, 4)),
    ('bispec', 'cic', 32, (2, 0, 2), 'off-diag', 1, (0.01, 0.1, 5)),
    ('bispec', 'pcs', 32, (2, 0, 2), 'row', 2, (0.01, 0.1, 4)),
    ('bispec', 'tsc', 32, (1, 1, 0), 'full', None, (0.01, 0.1, 3)),
    ('bispec', 'tsc', 32, (1, 1, 2), 'diag', None, (0.01, 0.1, 3)),
    ('bispec', 'tsc', 32, (2, 2, 0), 'diag', None, (0.01, 0.1, 3)),
    # pruned evaluation grid (4K + 1 < N)
    ('bispec', 'tsc', 64, (0, 0, 0), 'diag', None, (0.005, 0.055, 5)),
    ('bispec', 'pcs', 64, (2, 0, 2), 'full', None, (0.005, 0.045, 4)),
    ('bispec', 'cic', 64, (1, 1, 2), 'full', None, (0.005, 0.045, 3)),
    ('3pcf', 'tsc', 32, (0, 0, 0), 'diag', None, (40., 160., 4)),
    ('3pcf', 'cic', 32, (2, 0, 2), 'row', 1, (40., 160., 4)),
    ('3pcf', 'tsc', 32, (1, 1, 0), 'full', None, (40., 160., 3)),
    # the large-mesh 3PCF's path (PCS, j_l-weighted fields on the full
    # mesh from the key table, zeta_110 diag) at 64^3
    ('3pcf', 'pcs', 64, (1, 1, 0), 'diag', None, (20., 150., 5)),
    ('3pcf', 'pcs', 64, (0, 0, 0), 'diag', None, (20., 150., 5)),
]


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("kind, assignment, ngrid, degrees, form, idx_bin, "
                         "bins", GPP_CASES)
def test_oracle_gpp(precision, kind, assignment, ngrid, degrees, form,
                    idx_bin, bins):
    box, n = 800., 3000
    pos = _uniform(n, box, seed=ngrid + sum(degrees) + len(form))
    ref = _oracle_gpp(kind, pos, box, ngrid, assignment, degrees, form,
                      idx_bin, bins)
    cat = ParticleCatalogue(pos[:, 0], pos[:, 1], pos[:, 2],
                            nz=n / box ** 3)
    space = 'fourier' if kind == 'bispec' else 'config'
    binning = Binning(space, 'lin', *bins)
    fn = compute_bispec_in_gpp_box if kind == 'bispec' \
        else compute_3pcf_in_gpp_box
    res = fn(cat, degrees=degrees, binning=binning, form=form,
             idx_bin=idx_bin,
             sampling_params=_sampling(precision, ngrid, assignment,
                                       box=box))
    assert_close_threept(res, ref, kind, precision,
                         fp32_rtol(kind, degrees))


def _survey_inputs(nd, nr, seed):
    rng = np.random.default_rng(seed)
    d = rng.uniform(-300., 300., size=(nd, 3)) + [0., 0., 800.]
    r = rng.uniform(-300., 300., size=(nr, 3)) + [0., 0., 800.]
    wd = rng.uniform(0.5, 1.5, nd)
    wr = rng.uniform(0.5, 1.5, nr)
    return d, r, wd, wr


def _oracle_survey(kind, d, r, wd, wr, box, ngrid, assignment, degrees,
                   form, idx_bin, bins, interlace=False):
    los_d = O.compute_los(*d.T)
    los_r = O.compute_los(*r.T)
    box3 = [box] * 3 if np.isscalar(box) else list(box)
    (dx, dy, dz), _ = O.centre(*d.T, box3, ref=tuple(r.T))
    (rx, ry, rz), _ = O.centre(*r.T, box3)
    data = dict(pos=np.stack([dx, dy, dz], -1), los=los_d, w=wd,
                ws=np.ones_like(wd))
    rand = dict(pos=np.stack([rx, ry, rz], -1), los=los_r, w=wr,
                ws=np.ones_like(wr))
    alpha = d.shape[0] / r.shape[0]
    npoint = '2pt' if kind == 'powspec' else '3pt'
    p = O.Params(box, ngrid, assignment, interlace, *degrees, form=form,
                 idx_bin=idx_bin, npoint=npoint)
    edges, centres = O.lin_binning(*bins)
    nz = np.full(r.shape[0], 1e-4)
    if kind == 'powspec':
        norm = O.powspec_norm_from_particles(nz, 1., wr, alpha)
        return O.compute_powspec(data, rand, p, edges, centres, norm)
    norm = O.bispec_norm_from_particles(nz, 1., wr, alpha)
    fn = O.compute_bispec if kind == 'bispec' else O.compute_3pcf
    return fn(data, rand, p, edges, centres, norm)


LPP_CASES = [
    ('bispec', 'tsc', 32, (0, 0, 0), 'diag', None, (0.01, 0.1, 4)),
    ('bispec', 'pcs', 32, (2, 0, 2), 'diag', None, (0.01, 0.1, 4)),
    ('bispec', 'cic', 32, (1, 1, 2), 'full', None, (0.01, 0.1, 3)),
    ('bispec', 'tsc', 64, (2, 0, 2), 'off-diag', -1, (0.005, 0.045, 4)),
    ('3pcf', 'tsc', 32, (2, 0, 2), 'diag', None, (40., 160., 4)),
    ('3pcf', 'cic', 32, (1, 1, 0), 'row', 0, (40., 160., 3)),
]


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("kind, assignment, ngrid, degrees, form, idx_bin, "
                         "bins", LPP_CASES)
def test_oracle_lpp(precision, kind, assignment, ngrid, degrees, form,
                    idx_bin, bins):
    box = 1000.
    d, r, wd, wr = _survey_inputs(1500, 6000, seed=ngrid + sum(degrees))
    ref = _oracle_survey(kind, d, r, wd, wr, box, ngrid, assignment,
                         degrees, form, idx_bin, bins)
    dc = ParticleCatalogue(*d.T, nz=1e-4, wc=wd)
    rc = ParticleCatalogue(*r.T, nz=1e-4, wc=wr)
    space = 'fourier' if kind == 'bispec' else 'config'
    fn = compute_bispec if kind == 'bispec' else compute_3pcf
    res = fn(dc, rc, degrees=degrees, binning=Binning(space, 'lin', *bins),
             form=form, idx_bin=idx_bin,
             sampling_params=_sampling(precision, ngrid, assignment,
                                       box=box))
    assert_close_threept(res, ref, kind, precision,
                         fp32_rtol(kind, degrees, survey=True))


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("assignment, interlace, ell",
                         [('tsc', True, 0), ('cic', True, 2),
                          ('pcs', False, 2), ('ngp', True, 0)])
def test_oracle_powspec(precision, assignment, interlace, ell):
    box, n, ngrid = 600., 4000, 32
    pos = _uniform(n, box, seed=5 + ell)
    bins = (0.01, 0.15, 6)
    x, y, z = O.periodise(*pos.T, [box] * 3)
    p = O.Params(box, ngrid, assignment, interlace, 0, 0, ell, npoint='2pt')
    edges, centres = O.lin_binning(*bins)
    norm = O.powspec_norm_from_particles(np.full(n, n / box ** 3), 1., 1.)
    ref = O.compute_powspec_in_gpp_box(np.stack([x, y, z], -1), p, edges,
                                       centres, norm)
    res = compute_powspec_in_gpp_box(
        ParticleCatalogue(*pos.T, nz=n / box ** 3), degree=ell,
        binning=Binning('fourier', 'lin', *bins),
        sampling_params=_sampling(precision, ngrid, assignment, interlace,
                                  box))
    assert np.array_equal(res['nmodes'], ref['nmodes'])
    assert rel_err(res['keff'], ref['keff']) < 1e-12
    _check_pk(res, ref, precision)

    d, r, wd, wr = _survey_inputs(1200, 5000, seed=11 + ell)
    ref = _oracle_survey('powspec', d, r, wd, wr, 1000., ngrid, assignment,
                         (0, 0, ell), 'diag', None, bins, interlace)
    res = compute_powspec(ParticleCatalogue(*d.T, nz=1e-4, wc=wd),
                          ParticleCatalogue(*r.T, nz=1e-4, wc=wr),
                          degree=ell,
                          binning=Binning('fourier', 'lin', *bins),
                          sampling_params=_sampling(precision, ngrid,
                                                    assignment, interlace,
                                                    1000.))
    assert np.array_equal(res['nmodes'], ref['nmodes'])
    _check_pk(res, ref, precision)


def _check_pk(res, ref, precision):
    """Shot noise of ell > 0 is zero up to rounding: it is compared on the
    scale of the raw multipole."""
    assert_close_vector(res['pk_raw'], ref['pk_raw'], precision, 'pk_raw')
    scale = float(np.max(np.abs(ref['pk_raw'])))
    tol = 1e-9 if precision == 'fp64' else 1e-5
    err = np.abs(res['pk_shot'] - ref['pk_shot'])
    assert np.all(err <= tol * np.abs(ref['pk_shot']) + tol * scale), \
        float(np.max(err) / scale)


# ---------------------------------------------------------------------------
# Mesh assignment (K1) against the oracle, mesh cell by mesh cell
# ---------------------------------------------------------------------------

@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("assignment", ['ngp', 'cic', 'tsc', 'pcs'])
@pytest.mark.parametrize("shadow", [False, True])
def test_assignment_mesh(precision, assignment, shadow):
    box, ngrid, n = 500., 16, 2500
    rng = np.random.default_rng(3)
    pos = rng.uniform(0., box, size=(n, 3))
    # Particles on cell boundaries and at the box edge exercise the wraps.
    pos[:8] = [[0., 0., 0.], [box * (1 - 1e-15), 0., 0.],
               [box / ngrid * 3, box / 2, 0.],
               [box / ngrid * 2.5, box / ngrid * 0.5, box / ngrid * 15.5],
               [box / ngrid * 15.5, 0., 0.], [box / ngrid * 14.5, 0., 1.],
               [box / ngrid * 15.999, 3., 7.], [1e-9, 1e-9, 1e-9]]
    w = rng.uniform(0.5, 2., n)
    p = O.Params(box, ngrid, assignment, True, npoint='2pt')
    ref = O.assign_weighted_field_to_mesh(pos, w.astype(complex), p,
                                          shadow=shadow).real
    ctx = _lib.default_context()
    pc = _engine.make_params({'boxsize': {'x': box, 'y': box, 'z': box},
                              'ngrid': {'x': ngrid, 'y': ngrid, 'z': ngrid},
                              'assignment_order': p.assignment_order,
                              'interlace': True, 'degrees': {},
                              'form': 'diag', 'precision': precision,
                              'verbose': 0}, '2pt')
    cat = _engine.HostCatalogue(pos[:, 0], pos[:, 1], pos[:, 2], w)
    mesh = _engine.assign_mesh(ctx, pc, cat.c, shadow=shadow)
    tol = 1e-12 if precision == 'fp64' else 1e-6
    assert np.max(np.abs(mesh - ref)) <= tol * np.max(np.abs(ref))
    assert abs(mesh.sum() - ref.sum()) <= tol * abs(ref.sum())


def test_mesh_norm_matches_oracle():
    box, ngrid, n = 500., 32, 3000
    pos = _uniform(n, box, 9)
    w = np.random.default_rng(9).uniform(0.5, 1.5, n)
    p = O.Params(box, ngrid, 'tsc', False)
    for order in (2, 3):
        ref = O.grid_powlaw_norm(pos, w, p, order)
        ctx = _lib.default_context()
        pc = _engine.make_params({'boxsize': {'x': box, 'y': box, 'z': box},
                                  'ngrid': {'x': ngrid, 'y': ngrid,
                                            'z': ngrid},
                                  'assignment_order': 3, 'interlace': False,
                                  'degrees': {}, 'form': 'diag',
                                  'precision': 'fp64', 'verbose': 0}, '2pt')
        cat = _engine.HostCatalogue(pos[:, 0], pos[:, 1], pos[:, 2], w)
        got = _engine.grid_powlaw_norm(ctx, pc, cat.c, order)
        assert abs(got / ref - 1.) < 1e-10


# ---------------------------------------------------------------------------
# Edge cases and errors
# ---------------------------------------------------------------------------

def test_vanishing_multipole_raises():
    cat = ParticleCatalogue(*_uniform(100, 500., 1).T, nz=1e-6)
    with pytest.raises(_lib.InvalidParameterError, match="Wigner 3-j"):
        compute_bispec_in_gpp_box(
            cat, degrees=(1, 0, 0), binning=Binning('fourier', 'lin', 0.01,
                                                    0.1, 3),
            form='diag', sampling_params=_sampling('fp64', 16, box=500.))


def test_empty_bin_gives_zero_modes_like_reference():
    """A bin below the fundamental mode has no modes: nmodes = 0 and k_eff
    = 0/0 as in field.cpp:1905."""
    cat = ParticleCatalogue(*_uniform(500, 1000., 2).T, nz=5e-7)
    res = compute_bispec_in_gpp_box(
        cat, degrees=(0, 0, 0),
        binning=Binning('fourier', 'lin', 0.0001, 0.0021, 2), form='diag',
        sampling_params=_sampling('fp64', 16))
    assert list(res['nmodes_1']) == [0, 0]
    assert np.all(np.isnan(res['k1_eff']))


def test_repeat_calls_are_reproducible():
    pos = _uniform(5000, 700., 4)
    out = []
    for _ in range(3):
        cat = ParticleCatalogue(*pos.T, nz=5000 / 700. ** 3)
        out.append(compute_bispec_in_gpp_box(
            cat, degrees=(0, 0, 0),
            binning=Binning('fourier', 'lin', 0.01, 0.1, 5), form='diag',
            sampling_params=_sampling('fp64', 32, box=700.)))
    for o in out[1:]:
        assert np.array_equal(o['nmodes_1'], out[0]['nmodes_1'])
        assert rel_err(o['bk_raw'], out[0]['bk_raw']) < 1e-12
        assert rel_err(o['bk_shot'], out[0]['bk_shot']) < 1e-12


def test_device_inputs_match_host_inputs():
    """Particle arrays already in device memory give the host result."""
    torch = pytest.importorskip("torch")
    box, n = 700., 4000
    pos = _uniform(n, box, 12)
    x, y, z = O.periodise(*pos.T, [box] * 3)
    ctx = _lib.default_context()
    pdict = {'boxsize': {'x': box, 'y': box, 'z': box},
             'ngrid': {'x': 32, 'y': 32, 'z': 32}, 'assignment_order': 3,
             'interlace': False, 'degrees': {'ell1': 0, 'ell2': 0, 'ELL': 0},
             'form': 'diag', 'shape': 'diag', 'precision': 'fp32mixed',
             'verbose': 0}
    pc = _engine.make_params(pdict, '3pt')
    binning = Binning('fourier', 'lin', 0.01, 0.1, 5)
    host = _engine.HostCatalogue(x, y, z)
    r1 = _engine.call_threept('trvg_compute_bispec_in_gpp_box', ctx, pc,
                              host.c, binning, 1., 'bispec', shape='diag')
    dev = [torch.as_tensor(a, dtype=torch.float64, device='cuda')
           for a in (x, y, z)]
    dc = _engine.device_catalogue(n, *(t.data_ptr() for t in dev))
    torch.cuda.synchronize()
    r2 = _engine.call_threept('trvg_compute_bispec_in_gpp_box', ctx, pc, dc,
                              binning, 1., 'bispec', shape='diag')
    assert np.array_equal(r1['nmodes_1'], r2['nmodes_1'])
    assert rel_err(r1['bk_raw'], r2['bk_raw']) < 1e-5


@pytest.mark.parametrize("boxsize, ngrid", [((800., 800., 1000.), (32, 32, 32)),
                                            ((700., 700., 700.), (27, 27, 27)),
                                            ((600., 700., 800.), (24, 28, 32))])
def test_oracle_gpp_noncubic_and_odd(boxsize, ngrid):
    """Non-cubic cells use the cell-by-cell Bessel sum, odd meshes the
    cell-by-cell histogram, unequal x/y meshes the orbit sum without the
    x <-> y swap."""
    n = 2500
    rng = np.random.default_rng(21)
    pos = rng.uniform(0., 1., size=(n, 3)) * np.array(boxsize)
    bins = (0.01, 0.1, 4)
    x, y, z = O.periodise(*pos.T, list(boxsize))
    p = O.Params(list(boxsize), list(ngrid), 'tsc', False, 0, 0, 0,
                 form='diag')
    edges, centres = O.lin_binning(*bins)
    vol = float(np.prod(boxsize))
    norm = O.bispec_norm_from_particles(np.full(n, n / vol), 1., 1.)
    ref = O.compute_bispec_in_gpp_box(np.stack([x, y, z], -1), p, edges,
                                      centres, norm)
    for precision in PRECISIONS:
        res = compute_bispec_in_gpp_box(
            ParticleCatalogue(*pos.T, nz=n / vol), degrees=(0, 0, 0),
            binning=Binning('fourier', 'lin', *bins), form='diag',
            sampling_params={'boxsize': list(boxsize), 'ngrid': list(ngrid),
                             'assignment': 'tsc', 'precision': precision})
        assert_close_threept(res, ref, 'bispec', precision)


@pytest.mark.parametrize("shell64, shot64", [(0, 1), (1, 0), (1, 1)])
def test_fp32mixed_precision_options(shell64, shot64):
    """The FP64 evaluation-grid / shot-noise options of the FP32-mixed path
    stay within its tolerance of the oracle."""
    box, n, ngrid = 800., 3000, 32
    pos = _uniform(n, box, seed=31)
    bins = (0.01, 0.1, 5)
    ref = _oracle_gpp('bispec', pos, box, ngrid, 'tsc', (2, 0, 2), 'diag',
                      None, bins)
    ctx = _lib.default_context()
    ctx.set_option('shell_fields_fp64', shell64)
    ctx.set_option('shotnoise_fp64', shot64)
    try:
        res = compute_bispec_in_gpp_box(
            ParticleCatalogue(*pos.T, nz=n / box ** 3), degrees=(2, 0, 2),
            binning=Binning('fourier', 'lin', *bins), form='diag',
            sampling_params=_sampling('fp32mixed', ngrid, box=box))
    finally:
        ctx.set_option('shell_fields_fp64', 0)
        ctx.set_option('shotnoise_fp64', 0)
    # These options evaluate fields from the FP32 spectrum of the mesh,
    # not the float-float transforms.
    assert_close_threept(res, ref, 'bispec', 'fp32mixed', RTOL_FP32_FFT)


@pytest.mark.parametrize("precision", PRECISIONS)
def test_oracle_gpp_sorted_catalogue(precision):
    """Catalogues of >= 65536 particles are tile-sorted on the device before
    assignment; the result must not change."""
    box, n, ngrid = 900., 100000, 32
    pos = _uniform(n, box, seed=77)
    bins = (0.01, 0.1, 4)
    ref = _oracle_gpp('bispec', pos, box, ngrid, 'pcs', (0, 0, 0), 'diag',
                      None, bins)
    res = compute_bispec_in_gpp_box(
        ParticleCatalogue(*pos.T, nz=n / box ** 3), degrees=(0, 0, 0),
        binning=Binning('fourier', 'lin', *bins), form='diag',
        sampling_params=_sampling(precision, ngrid, 'pcs', box=box))
    assert_close_threept(res, ref, 'bispec', precision)


def test_oracle_lpp_sorted_randoms():
    d, r, wd, wr = _survey_inputs(2000, 80000, seed=78)
    bins = (0.01, 0.1, 3)
    ref = _oracle_survey('bispec', d, r, wd, wr, 1000., 32, 'tsc', (2, 0, 2),
                         'diag', None, bins)
    res = compute_bispec(ParticleCatalogue(*d.T, nz=1e-4, wc=wd),
                         ParticleCatalogue(*r.T, nz=1e-4, wc=wr),
                         degrees=(2, 0, 2),
                         binning=Binning('fourier', 'lin', *bins), form='diag',
                         sampling_params=_sampling('fp64', 32, 'tsc',
                                                   box=1000.))
    assert_close_threept(res, ref, 'bispec', 'fp64')


# ---------------------------------------------------------------------------
# Measurement files written by the estimators
# ---------------------------------------------------------------------------

@pytest.mark.parametrize("stat", ['bispec', 'powspec'])
def test_save_writes_readable_measurements(stat, tmp_path):
    from triumvirate_gb300 import io
    from triumvirate_gb300.twopt import compute_powspec_in_gpp_box
    from triumvirate_gb300.parameters import (ParameterSet,
                                              fetch_paramset_template)
    pos = _uniform(3000, 800., 13)
    cat = ParticleCatalogue(*pos.T, nz=3000 / 800. ** 3)
    d = fetch_paramset_template('dict')
    d.update(boxsize={ax: 800. for ax in 'xyz'},
             ngrid={ax: 32 for ax in 'xyz'}, assignment='tsc',
             interlace=False, precision='fp64')
    d['directories']['measurements'] = str(tmp_path)
    binning = Binning('fourier', 'lin', 0.01, 0.1, 4)
    if stat == 'bispec':
        res = compute_bispec_in_gpp_box(
            cat, degrees=(0, 0, 0), binning=binning, form='diag',
            paramset=ParameterSet(param_dict=d), save='.txt')
        path, raw = tmp_path / 'bk000_diag.txt', 'bk_raw'
    else:
        res = compute_powspec_in_gpp_box(
            cat, degree=0, binning=binning,
            paramset=ParameterSet(param_dict=d), save='.txt')
        path, raw = tmp_path / 'pk0.txt', 'pk_raw'
    back = io.read_measurements(path)
    assert np.allclose(back[raw], res[raw], rtol=1e-9, atol=0.)
    alt = next(h for h in back['header']
               if h.startswith('Normalisation factor alternatives'))
    mesh = float(alt.split(', ')[1].split(' (')[0])
    assert np.isfinite(mesh) and mesh > 0.


# ---------------------------------------------------------------------------
# Batched catalogues
# ---------------------------------------------------------------------------

@pytest.mark.parametrize("precision", ['fp64', 'fp32mixed'])
def test_batch_matches_single_calls(precision):
    """Mocks of uneven sizes in one call give each mock's own result."""
    from triumvirate_gb300.threept import compute_bispec_in_gpp_box_batch
    box, sizes = 600., [1500, 4000, 2500]
    pos = [_uniform(n, box, 30 + i) for i, n in enumerate(sizes)]
    binning = Binning('fourier', 'lin', 0.01, 0.1, 4)
    samp = _sampling(precision, 32, box=box)

    def cats():
        return [ParticleCatalogue(*p.T, nz=len(p) / box ** 3) for p in pos]
    single = [compute_bispec_in_gpp_box(c, degrees=(0, 0, 0),
                                        binning=binning, form='diag',
                                        sampling_params=samp)
              for c in cats()]
    batch = compute_bispec_in_gpp_box_batch(cats(), degrees=(0, 0, 0),
                                            binning=binning, form='diag',
                                            sampling_params=samp)
    assert len(batch) == len(single)
    for b, s in zip(batch, single):
        assert np.array_equal(b['nmodes_1'], s['nmodes_1'])
        for k in ('bk_raw', 'bk_shot'):
            if precision == 'fp64':
                assert rel_err(b[k], s[k]) < 1e-10, k
            else:
                # FP32 atomics deposit in a different order on each call.
                assert_per_bin(b[k], s[k], k, 2 * RTOL_FP32)


@pytest.mark.parametrize("degrees", [(0, 0, 0), (2, 0, 2)])
def test_batch_graph_replay_matches_single_calls(degrees):
    """FP32-mixed batch on the float-float path (64^3, pruned grid M = 36):
    the largest mock runs as a warm-up, the others replay one captured CUDA
    graph with per-mock counts and offsets read on the device (sorted and
    unsorted sizes), and every mock matches its own single call and FP64."""
    from triumvirate_gb300.threept import compute_bispec_in_gpp_box_batch
    box, sizes = 1000., [70000, 30000, 90000, 50000]
    pos = [_uniform(n, box, 50 + i) for i, n in enumerate(sizes)]
    binning = Binning('fourier', 'lin', 0.005, 0.045, 4)

    def cats():
        return [ParticleCatalogue(*q.T, nz=len(q) / box ** 3) for q in pos]
    kw = dict(degrees=degrees, binning=binning, form='diag')
    batch = compute_bispec_in_gpp_box_batch(
        cats(), sampling_params=_sampling('fp32mixed', 64, box=box), **kw)
    assert _lib.default_context(None).stats()['graph_replays'] == 3
    for i, c in enumerate(cats()):
        s32 = compute_bispec_in_gpp_box(
            c, sampling_params=_sampling('fp32mixed', 64, box=box), **kw)
        s64 = compute_bispec_in_gpp_box(
            c, sampling_params=_sampling('fp64', 64, box=box), **kw)
        b = batch[i]
        assert np.array_equal(b['nmodes_1'], s64['nmodes_1'])
        assert np.allclose(b['k1_eff'], s64['k1_eff'], rtol=1e-12, atol=0)
        for k in ('bk_raw', 'bk_shot'):
            assert_per_bin(b[k], s32[k], (i, k), 2 * RTOL_FP32)
            assert_per_bin(b[k], s64[k], (i, k))


def test_autotuner_picks_candidates_and_keeps_results():
    """The tuned sort tile and pair bin batch come from their candidate
    sets and change nothing beyond FP32 deposit order."""
    box = 1000.
    cat = ParticleCatalogue(*_uniform(80000, box, 7).T, nz=80000 / box ** 3)
    kw = dict(degrees=(0, 0, 0), form='diag',
              binning=Binning('fourier', 'lin', 0.005, 0.045, 4),
              sampling_params=_sampling('fp32mixed', 64, box=box))
    ctx = _lib.default_context(None)
    ctx.set_option('autotune', 0)
    ctx.set_option('autotune', 1)
    tuned_res = compute_bispec_in_gpp_box(cat, **kw)
    tuned = ctx.tuned()
    tiles = [v for k, v in tuned.items() if k.startswith('sort_tile_shift')]
    batches = [v for k, v in tuned.items() if k.startswith('pair_bin_batch')]
    assert tiles and set(tiles) <= {2, 3, 4, 5}
    assert batches and set(batches) <= {4, 8, 16}
    ctx.set_option('autotune', 0)
    try:
        plain = compute_bispec_in_gpp_box(cat, **kw)
    finally:
        ctx.set_option('autotune', 1)
    for k in ('bk_raw', 'bk_shot'):
        assert_per_bin(tuned_res[k], plain[k], k, 2 * RTOL_FP32)


# ---------------------------------------------------------------------------
# Float-float shell-field transforms (FP32-mixed default)
# ---------------------------------------------------------------------------

@pytest.mark.parametrize("bins", [(0.005, 0.045, 4), (0.005, 0.05, 4),
                                  (0.005, 0.065, 4)])
@pytest.mark.parametrize("degrees, form", [((0, 0, 0), 'diag'),
                                           ((2, 0, 2), 'full')])
def test_float_float_transforms_match_fp64(bins, degrees, form):
    """Evaluation grids M = 25 (odd, the G band filling the grid), 30 and
    40: FP32-mixed with float-float transforms agrees with FP64 to 1e-6
    normwise and 1e-5 per entry, and is no less accurate than FP32
    transforms.  The mesh is deposited compensated (mesh_comp = 1), so
    that the comparison isolates the transforms from the FP32 deposit of
    this sparse catalogue (3000 particles on 64^3)."""
    box, n = 800., 3000
    pos = _uniform(n, box, seed=80)
    binning = Binning('fourier', 'lin', *bins)
    ctx = _lib.default_context()

    def run(precision, ff=1):
        ctx.set_option('ff_transforms', ff)
        ctx.set_option('mesh_comp', 1)
        try:
            cat = ParticleCatalogue(*pos.T, nz=n / box ** 3)
            return compute_bispec_in_gpp_box(
                cat, degrees=degrees, binning=binning, form=form,
                sampling_params=_sampling(precision, 64, box=box))['bk_raw']
        finally:
            ctx.set_option('ff_transforms', 1)
            ctx.set_option('mesh_comp', 2)
    ref = run('fp64')
    scale = np.max(np.abs(ref))
    ff = run('fp32mixed')
    err_ff = np.max(np.abs(ff - ref)) / scale
    err_32 = np.max(np.abs(run('fp32mixed', 0) - ref)) / scale
    assert_per_bin(ff, ref, 'bk_raw')
    assert err_ff < 1e-6, err_ff
    assert err_ff < 2. * err_32 + 1e-7, (err_ff, err_32)
    # Forward transform only in float-float (FP32 inverse transforms).
    fwd = run('fp32mixed', 2)
    err_fwd = np.max(np.abs(fwd - ref)) / scale
    assert err_fwd < 1e-6, (err_fwd, err_32)
    assert_per_bin(fwd, ref, 'bk_raw', RTOL_FP32_FFT)


@pytest.mark.parametrize("degrees", [(0, 0, 0), (2, 0, 2)])
def test_float_float_path_on_non_cubic_mesh(degrees):
    """A cubic box on a 64 x 48 x 80 mesh keeps the float-float shell fields
    (one band K on all axes, M = 30 below every mesh axis; forward passes
    over lines of 64, 48 and 80 points), while its cells are not cubic, so
    the shot-noise field is the full-mesh one (the octant form and the
    z-pass planes need cubic cells, i.e. a cubic mesh here): both agree
    with FP64 per bin."""
    box, n = 800., 60000
    pos = _uniform(n, box, seed=91)
    binning = Binning('fourier', 'lin', 0.005, 0.05, 5)

    def run(precision):
        cat = ParticleCatalogue(*pos.T, nz=n / box ** 3)
        return compute_bispec_in_gpp_box(
            cat, degrees=degrees, binning=binning, form='diag',
            sampling_params=_sampling(precision, [64, 48, 80], box=box))
    got, ref = run('fp32mixed'), run('fp64')
    assert np.array_equal(got['nmodes_1'], ref['nmodes_1'])
    for k in ('bk_raw', 'bk_shot'):
        scale = np.max(np.abs(ref[k]))
        assert np.max(np.abs(got[k] - ref[k])) <= 1e-6 * scale, (
            k, float(np.max(np.abs(got[k] - ref[k])) / scale))
        assert_per_bin(got[k], ref[k], k, RTOL_FP32_FFT)


# ---------------------------------------------------------------------------
# Shared-memory tiled deposit (32^3 tiles) against the oracle and the
# per-particle atomic deposit
# ---------------------------------------------------------------------------

def _with_assign_path(ctx, path, fn):
    ctx.set_option('assign_path', path)
    try:
        return fn()
    finally:
        ctx.set_option('assign_path', 0)


@pytest.mark.parametrize("assignment", ['ngp', 'cic', 'tsc', 'pcs'])
@pytest.mark.parametrize("box, ngrid", [(500., [64, 64, 64]),
                                        ([450., 600., 520.], [70, 96, 68]),
                                        ([450., 600., 520.], [70, 96, 65])])
def test_tiled_assignment_matches_oracle(assignment, box, ngrid):
    """Sorted catalogues (>= 65536 particles) of an FP32 mesh deposit tile
    by tile through shared memory; particles on cell edges, half cells and
    the box edge take the deferred exact path.  Partial tiles in x and z
    (70, 96, 68 cells) and every stencil order are covered; with 65 cells
    along z the rows are not 16-byte aligned and the atomic deposit is
    used instead."""
    boxv = np.array([box] * 3 if np.isscalar(box) else box, dtype=float)
    n = 70000
    rng = np.random.default_rng(17)
    pos = rng.uniform(0., 1., size=(n, 3)) * boxv
    cell = boxv / np.array(ngrid)
    k = rng.integers(0, 64, size=(300, 3))
    pos[:300] = k * cell                          # on cell edges
    pos[300:600] = (k + 0.5) * cell               # on half cells
    pos[600:603] = boxv * (1 - 1e-15)             # at the upper box edge
    pos[603:640] = (np.array(ngrid) - 1) * cell + rng.uniform(
        0., 1., (37, 3)) * cell                   # last cells: periodic wrap
    w = rng.uniform(0.5, 2., n)
    p = O.Params(boxv, ngrid, assignment, False, npoint='2pt')
    ref = O.assign_weighted_field_to_mesh(pos, w.astype(complex), p).real
    ctx = _lib.default_context()
    pc = _engine.make_params({'boxsize': dict(zip('xyz', boxv)),
                              'ngrid': dict(zip('xyz', ngrid)),
                              'assignment_order': p.assignment_order,
                              'interlace': False, 'degrees': {},
                              'form': 'diag', 'precision': 'fp32mixed',
                              'verbose': 0}, '2pt')
    cat = _engine.HostCatalogue(pos[:, 0], pos[:, 1], pos[:, 2], w)
    tiled = _with_assign_path(
        ctx, 1, lambda: _engine.assign_mesh(ctx, pc, cat.c))
    atomic = _with_assign_path(
        ctx, 2, lambda: _engine.assign_mesh(ctx, pc, cat.c))
    scale = np.max(np.abs(ref))
    assert np.max(np.abs(tiled - ref)) <= 1e-6 * scale
    assert np.max(np.abs(tiled - atomic)) <= 1e-6 * scale
    assert abs(tiled.sum() - ref.sum()) <= 1e-6 * abs(ref.sum())


@pytest.mark.parametrize("assignment", ['tsc', 'pcs'])
def test_tiled_assignment_in_estimators(assignment, rand_catalogue_array):
    """Periodic box (the first deposit stores the cells only its tile
    reaches over the mean offset) and survey (data then randoms: the second
    deposit adds) agree between the tiled and atomic deposits."""
    box = 1000.
    d = _uniform(90000, box, 23)
    samp = _sampling('fp32mixed', 64, assignment=assignment, box=box)
    kw = dict(degrees=(0, 0, 0), form='diag',
              binning=Binning('fourier', 'lin', 0.005, 0.105, 5),
              sampling_params=samp)
    ctx = _lib.default_context(None)

    def gpp():
        return compute_bispec_in_gpp_box(
            ParticleCatalogue(*d.T, nz=len(d) / box ** 3), **kw)
    r = rand_catalogue_array
    rr = np.concatenate([r[:, :3], _uniform(60000, box, 24) - box / 2])

    def lpp():
        return compute_bispec(
            ParticleCatalogue(*(d - box / 2).T, nz=3e-9),
            ParticleCatalogue(*rr.T, nz=3e-9), **kw)
    # FP32 atomics deposit in a different order in the two paths (the
    # survey field nearly cancels data against randoms): 1e-5 of the
    # largest entry, the FP32-mixed contract.
    for fn in (gpp, lpp):
        t = _with_assign_path(ctx, 1, fn)
        a = _with_assign_path(ctx, 2, fn)
        for k in ('bk_raw', 'bk_shot'):
            assert_per_bin(t[k], a[k], (fn.__name__, k), 2 * RTOL_FP32)


# ---------------------------------------------------------------------------
# Y_lm-weighted fields of every order in one fused pass
# ---------------------------------------------------------------------------

@pytest.mark.parametrize("degrees, assignment", [((2, 0, 2), 'tsc'),
                                                 ((2, 2, 4), 'pcs'),
                                                 ((1, 1, 0), 'cic')])
def test_fused_ylm_fields_match_one_by_one(degrees, assignment,
                                           rand_catalogue_array):
    """Survey bispectrum, 3PCF and 3PCF window with every Y_lm-weighted
    field built by one weight-sum and one deposit pass per catalogue (FP32
    meshes) against the fields built one order at a time.  B_224 has nine
    orders M (27 targets, two fused passes)."""
    rng = np.random.default_rng(31)
    d = rng.uniform(-500., 500., size=(5000, 3))
    r = rand_catalogue_array
    ctx = _lib.default_context(None)
    samp = _sampling('fp32mixed', 32, assignment=assignment)
    kb = Binning('fourier', 'lin', 0.01, 0.1, 3)
    rb = Binning('config', 'lin', 60., 160., 3)

    def cats():
        return (ParticleCatalogue(*d.T, nz=3e-9),
                ParticleCatalogue(r[:, 0], r[:, 1], r[:, 2], nz=r[:, 3]))

    def run(fused):
        ctx.set_option('fused_ylm', fused)
        try:
            dc, rc = cats()
            b = compute_bispec(dc, rc, degrees=degrees, binning=kb,
                               form='full', sampling_params=samp)
            dc, rc = cats()
            z = compute_3pcf(dc, rc, degrees=degrees, binning=rb,
                             form='diag', sampling_params=samp)
            _, rc = cats()
            w = compute_3pcf_window(rc, degrees=degrees, binning=rb,
                                    form='diag', sampling_params=samp)
        finally:
            ctx.set_option('fused_ylm', 1)
        return b, z, w
    fb, fz, fw = run(1)
    sb, sz, sw = run(0)
    # FP32 atomics deposit in a different order on every run; a wrong order
    # M, power or conjugation would differ at O(1).
    for a, b, keys in [(fb, sb, ('bk_raw', 'bk_shot')),
                       (fz, sz, ('zeta_raw', 'zeta_shot')),
                       (fw, sw, ('zeta_raw', 'zeta_shot'))]:
        for k in keys:
            assert_per_bin(a[k], b[k], k, 2 * RTOL_FP32)


# ---------------------------------------------------------------------------
# Shot-noise field on one octant (three DCT-I passes)
# ---------------------------------------------------------------------------

@pytest.mark.parametrize("degrees", [(0, 0, 0), (2, 0, 2)])
@pytest.mark.parametrize("box, ngrid", [(1000., [64, 64, 64]),
                                        ([900., 900., 720.], [60, 60, 48])])
def test_octant_shot_noise_matches_full_mesh(degrees, box, ngrid):
    """FP32 periodic-box bispectra with the flip-averaged shot-noise field
    on the octant equal those with the full-mesh field, and the FP64
    oracle within the FP32-mixed tolerance."""
    boxv = [box] * 3 if np.isscalar(box) else box
    pos = _uniform(60000, 1., 41) * np.array(boxv)
    kw = dict(degrees=degrees, form='diag',
              binning=Binning('fourier', 'lin', 0.01, 0.13, 6),
              sampling_params={'boxsize': boxv, 'ngrid': ngrid,
                               'assignment': 'tsc', 'interlace': False,
                               'precision': 'fp32mixed'})
    ctx = _lib.default_context(None)

    def run(octant):
        ctx.set_option('xi_octant', octant)
        try:
            return compute_bispec_in_gpp_box(
                ParticleCatalogue(*pos.T, nz=len(pos) / np.prod(boxv)), **kw)
        finally:
            ctx.set_option('xi_octant', 1)
    o, f = run(1), run(0)
    # Both calls deposit the FP32 mesh with atomics (in a different order,
    # and the first may autotune the deposit): 1e-5 of the largest entry.
    for k in ('bk_raw', 'bk_shot'):
        assert_per_bin(o[k], f[k], k, 2 * RTOL_FP32)



@pytest.mark.parametrize("precision", PRECISIONS)
def test_oracle_lpp_unequal_cells(precision):
    """Survey bispectrum on cells of unequal sides (the shot-noise sums keyed
    by (|s_x|, |s_y|, |s_z|) with a radius table, y_a y_b of nonzero
    orders M) against the oracle."""
    box, ngrid = [900., 1000., 800.], [32, 36, 28]
    d, r, wd, wr = _survey_inputs(1500, 6000, seed=91)
    bins = (0.01, 0.1, 3)
    ref = _oracle_survey('bispec', d, r, wd, wr, box, ngrid, 'tsc',
                         (2, 0, 2), 'full', None, bins)
    res = compute_bispec(ParticleCatalogue(*d.T, nz=1e-4, wc=wd),
                         ParticleCatalogue(*r.T, nz=1e-4, wc=wr),
                         degrees=(2, 0, 2),
                         binning=Binning('fourier', 'lin', *bins), form='full',
                         sampling_params=_sampling(precision, ngrid, 'tsc',
                                                   box=box))
    assert_close_threept(res, ref, 'bispec', precision, RTOL_FP32_FFT)


def test_side_stream_shot_noise_matches_one_stream():
    """The periodic-box bispectrum with its shot-noise field on the second
    stream (next to the float-float shell fields) equals the one-stream
    estimate and the FP64 one within the FP32-mixed tolerance."""
    box = 1000.
    pos = _uniform(200000, box, 61)
    kw = dict(degrees=(0, 0, 0), form='diag',
              binning=Binning('fourier', 'lin', 0.005, 0.105, 8))
    ctx = _lib.default_context(None)

    def run(overlap, precision='fp32mixed'):
        ctx.set_option('overlap', overlap)
        try:
            return compute_bispec_in_gpp_box(
                ParticleCatalogue(*pos.T, nz=len(pos) / box ** 3),
                sampling_params=_sampling(precision, 128, box=box), **kw)
        finally:
            ctx.set_option('overlap', 1)
    two, one, ref = run(1), run(0), run(1, 'fp64')
    for k in ('bk_raw', 'bk_shot'):
        assert_per_bin(two[k], one[k], k, 2 * RTOL_FP32)
        assert_per_bin(two[k], ref[k], k)


# ---------------------------------------------------------------------------
# Register-tiled Gram form of the FP32 pair sums
# ---------------------------------------------------------------------------

@pytest.mark.parametrize("case", ['survey_b202_full', 'gpp_b000_full_fp32fft',
                                  'gpp_b202_full_fp32fft', 'gpp_zeta000_diag',
                                  'gpp_zeta110_full', 'gpp_b000_full_36bins',
                                  'gpp_b202_full_36bins',
                                  'gpp_b000_full_ff_36bins',
                                  'gpp_b202_full_ff_36bins',
                                  'gpp_b220_diag'])
def test_tiled_gram_matches_per_pair(case, rand_catalogue_array):
    """FP32 pair sums in the register-tiled Gram form (complex survey fields,
    real periodic-box fields with FP32 transforms, the hi words of
    float-float fields, the 3PCF's j_l-weighted fields) equal the
    one-entry-per-thread form (float-float products for float-float
    fields); forms full, triu and diag exercise tiles that hold one, some
    and all of their field pairs, and the 36-bin cases stage more than 64
    rows per chunk.  B_220 diag: legs of orders m and -m read one set of
    fields, leg b conjugated, against leg b transformed (the per-pair
    form)."""
    ctx = _lib.default_context(None)
    rng = np.random.default_rng(71)
    pos = rng.uniform(0., 800., size=(20000, 3))
    d = rng.uniform(-500., 500., size=(5000, 3))
    r = rand_catalogue_array
    kb = Binning('fourier', 'lin', 0.01, 0.12, 11)
    ff = case.endswith('ff_36bins')
    if case.endswith('36bins'):
        # Float-float transforms need an evaluation grid below the mesh:
        # 160^3, k < 0.28 h/Mpc gives M = 150.
        kb = Binning('fourier', 'lin', 0.005, 0.28 if ff else 0.3, 36)
    rb = Binning('config', 'lin', 40., 160., 6)

    def est():
        if case == 'survey_b202_full':
            return compute_bispec(
                ParticleCatalogue(*d.T, nz=3e-9),
                ParticleCatalogue(r[:, 0], r[:, 1], r[:, 2], nz=r[:, 3]),
                degrees=(2, 0, 2), binning=kb, form='full',
                sampling_params=_sampling('fp32mixed', 32, 'pcs'))
        cat = ParticleCatalogue(*pos.T, nz=len(pos) / 800. ** 3)
        samp = _sampling('fp32mixed', 160 if ff else
                         96 if case.endswith('36bins') else 48,
                         'tsc', box=800.)
        if case.startswith('gpp_b'):
            deg = ((0, 0, 0) if 'b000' in case else
                   (2, 2, 0) if 'b220' in case else (2, 0, 2))
            return compute_bispec_in_gpp_box(
                cat, degrees=deg, binning=kb,
                form='diag' if case.endswith('diag') else 'full',
                sampling_params=samp)
        deg = (0, 0, 0) if 'zeta000' in case else (1, 1, 0)
        form = 'diag' if 'diag' in case else 'full'
        return compute_3pcf_in_gpp_box(cat, degrees=deg, binning=rb,
                                       form=form, sampling_params=samp)

    def run(per_pair, transforms=1 if ff else 0):
        # Compensated, renormalised deposits: both runs transform the same
        # correctly rounded FP32 meshes whatever the order of the atomics.
        ctx.set_option('gram_per_pair', per_pair)
        ctx.set_option('ff_transforms', transforms)
        ctx.set_option('mesh_comp', 1)
        ctx.set_option('mesh_renorm', 1)
        try:
            return est()
        finally:
            ctx.set_option('gram_per_pair', 0)
            ctx.set_option('ff_transforms', 1)
            ctx.set_option('mesh_comp', 2)
            ctx.set_option('mesh_renorm', 0)
    tiled, pair = run(0), run(1)
    keys = ('bk_raw', 'bk_shot') if 'zeta' not in case \
        else ('zeta_raw', 'zeta_shot')
    # The forms differ in the FP32 partial sums of the tiled one (and, for
    # float-float fields, in the rounding of the fields to FP32): per entry
    # within 1e-5 for B_000 and the FP32-FFT bound otherwise, normwise to
    # 2e-6 (a wrong tile or slot would differ at O(1)).  B_202 has entries
    # near 1e-5 of the largest whose FP32 sums cancel; there both forms lie
    # some 3e-3 from FP64 and 5e-4 from each other, so its per-entry check
    # (and B_220's) covers the entries above 1e-3 of the largest.
    rtol = RTOL_FP32 if 'b000' in case else RTOL_FP32_FFT
    floor = 1e-3 if ('b202' in case or 'b220' in case) else 0.
    for k in keys:
        t, q = np.asarray(tiled[k]), np.asarray(pair[k])
        scale = np.max(np.abs(q))
        big = np.abs(q) >= floor * scale
        assert_per_bin(t[big], q[big], (case, k), rtol)
        assert np.max(np.abs(t - q)) <= 2e-6 * scale, (
            case, k, float(np.max(np.abs(t - q)) / scale))
    if ff:
        # The float-float transforms were taken: FP32 transforms give other
        # values.
        assert not np.array_equal(np.asarray(tiled['bk_raw']),
                                  np.asarray(run(0, 0)['bk_raw']))


def test_tiled_gram_complex_then_real_in_fresh_process():
    """A fresh process whose first tiled reduction is complex and whose next
    one is real (survey B_202: terms of order M != 0, then M = 0) opts both
    kernels in to their shared memory."""
    import subprocess
    import sys
    code = (
        "import numpy as np\n"
        "from triumvirate_gb300.catalogue import ParticleCatalogue\n"
        "from triumvirate_gb300.dataobjs import Binning\n"
        "from triumvirate_gb300.threept import compute_bispec\n"
        "rng = np.random.default_rng(5)\n"
        "d = rng.uniform(-300., 300., size=(3000, 3)) + [0., 0., 800.]\n"
        "r = rng.uniform(-300., 300., size=(12000, 3)) + [0., 0., 800.]\n"
        "res = compute_bispec(ParticleCatalogue(*d.T, nz=1e-4),\n"
        "                     ParticleCatalogue(*r.T, nz=1e-4),\n"
        "                     degrees=(2, 0, 2),\n"
        "                     binning=Binning('fourier', 'lin', 0.01, 0.1, 6),\n"
        "                     form='full',\n"
        "                     sampling_params={'boxsize': [1000.] * 3,\n"
        "                                      'ngrid': [32] * 3,\n"
        "                                      'assignment': 'tsc',\n"
        "                                      'precision': 'fp32mixed'})\n"
        "assert np.all(np.isfinite(res['bk_raw']))\n")
    import os
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    p = subprocess.run([sys.executable, "-c", code], cwd=root,
                       capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
