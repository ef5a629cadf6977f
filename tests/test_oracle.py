"""The CPU oracle against the reference's golden measurement files.

Tolerances are the reference tests' own (tests/test_threept.py:49-75,
tests/test_twopt.py:39-52): ``np.allclose`` defaults, plus ``atol=1e-6``
on shot noise.
"""
import os
from pathlib import Path

import numpy as np
import pytest

from conftest import BOX, KBINS, NMESH, RBINS, THREEPT_CASES, load_golden
from oracle import trv_oracle as O


def _gpp_pos(d):
    x, y, z = O.periodise(d[:, 0], d[:, 1], d[:, 2], [BOX] * 3)
    return np.stack([x, y, z], -1)


def _survey(d, r):
    los_d = O.compute_los(d[:, 0], d[:, 1], d[:, 2])
    los_r = O.compute_los(r[:, 0], r[:, 1], r[:, 2])
    ref = (r[:, 0], r[:, 1], r[:, 2])
    (dx, dy, dz), _ = O.centre(d[:, 0], d[:, 1], d[:, 2], [BOX] * 3, ref=ref)
    (rx, ry, rz), _ = O.centre(*ref, [BOX] * 3)
    nd, nr = d.shape[0], r.shape[0]
    data = dict(pos=np.stack([dx, dy, dz], -1), los=los_d, w=np.ones(nd),
                ws=np.ones(nd))
    rand = dict(pos=np.stack([rx, ry, rz], -1), los=los_r, w=np.ones(nr),
                ws=np.ones(nr))
    return data, rand, nd / nr


def check_threept(res, ext, kind, rtol=1e-5):
    keys = (['k1_bin', 'k1_eff', 'nmodes_1', 'k2_bin', 'k2_eff', 'nmodes_2',
             'bk_raw', 'bk_shot'] if kind == 'bispec' else
            ['r1_bin', 'r1_eff', 'npairs_1', 'r2_bin', 'r2_eff', 'npairs_2',
             'zeta_raw', 'zeta_shot'])
    for i, k in enumerate(keys[:6]):
        assert np.allclose(res[k], ext[i]), k
    assert np.allclose(res[keys[6]], ext[-4] + 1j * ext[-3], rtol=rtol), \
        keys[6]
    assert np.allclose(res[keys[7]], ext[-2] + 1j * ext[-1], rtol=rtol,
                       atol=1e-6), keys[7]


def check_powspec(res, ext):
    assert np.allclose(res['kbin'], ext[0])
    assert np.allclose(res['keff'], ext[1])
    assert np.allclose(res['nmodes'], ext[2])
    assert np.allclose(res['pk_raw'], ext[3] + 1j * ext[4])
    assert np.allclose(res['pk_shot'], ext[5] + 1j * ext[6], atol=1e-6)


@pytest.mark.parametrize("kind, degrees, form, idx_bin, golden",
                         THREEPT_CASES)
def test_oracle_gpp(kind, degrees, form, idx_bin, golden,
                    data_catalogue_array):
    d = data_catalogue_array
    p = O.Params(BOX, NMESH, 'tsc', False, *degrees, form=form,
                 idx_bin=idx_bin)
    bins = KBINS if kind == 'bispec' else RBINS
    edges, centres = O.lin_binning(*bins)
    norm = O.bispec_norm_from_particles(d[:, 3], 1., 1.)
    fn = (O.compute_bispec_in_gpp_box if kind == 'bispec'
          else O.compute_3pcf_in_gpp_box)
    res = fn(_gpp_pos(d), p, edges, centres, norm)
    check_threept(res, load_golden(golden.format('gpp')), kind)


@pytest.mark.parametrize("kind, degrees, form, idx_bin, golden",
                         THREEPT_CASES)
def test_oracle_lpp(kind, degrees, form, idx_bin, golden,
                    data_catalogue_array, rand_catalogue_array):
    data, rand, alpha = _survey(data_catalogue_array, rand_catalogue_array)
    p = O.Params(BOX, NMESH, 'tsc', False, *degrees, form=form,
                 idx_bin=idx_bin)
    bins = KBINS if kind == 'bispec' else RBINS
    edges, centres = O.lin_binning(*bins)
    norm = O.bispec_norm_from_particles(rand_catalogue_array[:, 3], 1., 1.,
                                        alpha)
    fn = O.compute_bispec if kind == 'bispec' else O.compute_3pcf
    res = fn(data, rand, p, edges, centres, norm)
    check_threept(res, load_golden(golden.format('lpp')), kind)


@pytest.mark.parametrize("ell", [0, 2])
def test_oracle_powspec(ell, data_catalogue_array, rand_catalogue_array):
    d = data_catalogue_array
    edges, centres = O.lin_binning(*KBINS)
    p = O.Params(BOX, NMESH, 'tsc', False, 0, 0, ell, npoint='2pt')
    norm = O.powspec_norm_from_particles(d[:, 3], 1., 1.)
    res = O.compute_powspec_in_gpp_box(_gpp_pos(d), p, edges, centres, norm)
    check_powspec(res, load_golden(f"pk{ell}_gpp.txt"))
    data, rand, alpha = _survey(d, rand_catalogue_array)
    norm = O.powspec_norm_from_particles(rand_catalogue_array[:, 3], 1., 1.,
                                         alpha)
    res = O.compute_powspec(data, rand, p, edges, centres, norm)
    check_powspec(res, load_golden(f"pk{ell}_lpp.txt"))


def test_random_catalogue_regeneration(rand_catalogue_array):
    """The regenerated randoms equal the reference's file bit for bit."""
    root = os.environ.get("TRIUMVIRATE_REFERENCE")
    if not root:
        pytest.skip("set TRIUMVIRATE_REFERENCE to the reference tree")
    f = Path(root) / "tests" / "test_input" / "ctlgs" / \
        "test_rand_catalogue.txt"
    ref = np.loadtxt(f)
    assert np.array_equal(ref, rand_catalogue_array)


def test_wigner_3j_exact():
    sympy = pytest.importorskip("sympy")
    from sympy.physics.wigner import wigner_3j
    for args in [(0, 0, 0, 0, 0, 0), (2, 0, 2, 0, 0, 0), (2, 0, 2, 1, 0, -1),
                 (1, 1, 2, 1, -1, 0), (3, 2, 1, -2, 1, 1),
                 (4, 4, 4, 2, -1, -1), (2, 2, 2, 0, 0, 0)]:
        assert abs(O.wigner_3j(*args) - float(wigner_3j(*args))) < 1e-15


WINDOW_CASES = [
    ((0, 0, 0), 'diag', None, 'zetaw000_diag.txt'),
    ((2, 0, 2), 'diag', None, 'zetaw202_diag.txt'),
    ((0, 0, 0), 'row', 0, 'zetaw000_row0.txt'),
]


def _window_rand(r):
    """The random catalogue as the reference's compute_3pcf_window prepares
    it (threept.py:1976-1987): lines of sight before centring, then
    centred and periodised in the box."""
    los = O.compute_los(r[:, 0], r[:, 1], r[:, 2])
    (x, y, z), _ = O.centre(r[:, 0], r[:, 1], r[:, 2], [BOX] * 3)
    x, y, z = O.periodise(x, y, z, [BOX] * 3)
    n = r.shape[0]
    return dict(pos=np.stack([x, y, z], -1), los=los, w=np.ones(n),
                ws=np.ones(n))


@pytest.mark.parametrize("degrees, form, idx_bin, golden", WINDOW_CASES)
def test_oracle_3pcf_window(degrees, form, idx_bin, golden,
                            rand_catalogue_array):
    rand = _window_rand(rand_catalogue_array)
    p = O.Params(BOX, NMESH, 'tsc', False, *degrees, form=form,
                 idx_bin=idx_bin)
    edges, centres = O.lin_binning(*RBINS)
    norm = O.bispec_norm_from_particles(rand_catalogue_array[:, 3], 1., 1.)
    res = O.compute_3pcf_window(rand, p, edges, centres, norm)
    check_threept(res, load_golden(golden), '3pcf')


def test_oracle_wide_angle_kernel():
    """r^-(i + j) away from the origin; orders (0, 0) leave G unchanged."""
    rng = np.random.default_rng(3)
    g = rng.normal(size=(4, 4, 4)) + 1j * rng.normal(size=(4, 4, 4))
    r = rng.uniform(1., 3., size=(4, 4, 4))
    r[0, 0, 0] = 0.
    out = O.wide_angle_pow_law(g, r, 1, 1)
    assert out[0, 0, 0] == g[0, 0, 0]
    far = r > 0
    assert np.allclose(out[far], g[far] / r[far] ** 2)
    assert np.array_equal(O.wide_angle_pow_law(g, r, 0, 0), g)


def test_bench_sample_entries_match_oracle_estimate():
    """The bench's bounded oracle sample (set-up + one bin pair) gives the
    same normalised diagonal entries as the oracle's whole B_000 estimate;
    it is the oracle check of the GPU estimate at the full workload size."""
    from oracle.sample import GppBispecSample
    npart, box, ngrid, nbins = 3000, 1000., 64, 20
    s = GppBispecSample(npart, box, ngrid, nbins, seed=5)
    s.setup()
    norm = O.bispec_norm_from_particles(np.full(npart, npart / box ** 3),
                                        1., 1.)
    p = O.Params(box, ngrid, 'tsc', False, 0, 0, 0, form='diag')
    ref = O.compute_bispec_in_gpp_box(s.pos, p, s.edges, s.centres, norm)
    for b in (0, nbins // 2):
        raw, shot, nm = s.entry(b, norm)
        assert nm == ref['nmodes_1'][b]
        assert abs(raw - ref['bk_raw'][b]) <= 1e-12 * abs(ref['bk_raw'][b])
        assert abs(shot - ref['bk_shot'][b]) <= 1e-12 * abs(ref['bk_shot'][b])
