"""GPU parity of device-resident catalogues (``trvg_dcat_*``).

* The multi-threaded text reader gives the same bits as ``np.loadtxt`` and
  as the oracle's restatement of ``load_catalogue_file``
  (particles.cpp:94-510), on the reference's own test catalogue and on
  synthetic files (comments, blank lines, tabs, CRLF, exponents, permuted
  and extra columns, "::"-joined sub-files).
* Periodising, centring, padding and lines of sight on the device give the
  same bits as ``ParticleCatalogue`` (numpy); the C-ABI padding and box
  folding give the same bits as the oracle's restatements of
  particles.cpp:678-888.  Weight totals and normalisation sums come from a
  fixed-order device reduction: relative 1e-13.
* Estimators fed device catalogues reproduce the reference's golden files
  and the host-catalogue results (relative 1e-12), with no particle copied
  from the host.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import BOX, GOLDEN, KBINS, NMESH, load_golden
from oracle import trv_oracle as O
from test_gpu_parity import _check_golden, _sampling, rel_err
from test_oracle import check_powspec
from triumvirate_gb300 import _lib
from triumvirate_gb300.catalogue import DeviceCatalogue, ParticleCatalogue
from triumvirate_gb300.dataobjs import Binning
from triumvirate_gb300.threept import (compute_bispec,
                                       compute_bispec_in_gpp_box,
                                       compute_bispec_in_gpp_box_batch)
from triumvirate_gb300.twopt import compute_powspec

pytestmark = pytest.mark.gpu

FORMATS = [repr, lambda v: f"{v:.6e}", lambda v: f"{v:+.3f}",
           lambda v: f"{v:.17g}", lambda v: f"{v:.2E}"]


def _write(path, rows, seed=0, crlf=False):
    """Rows with mixed number formats, separators and comment lines."""
    rng = np.random.default_rng(seed)
    out = ["# header line"]
    for i, row in enumerate(rows):
        fmt = FORMATS[int(rng.integers(len(FORMATS)))]
        sep = ["  ", "\t", " \t "][i % 3]
        out.append(sep.join(fmt(float(v)) for v in row))
        if i % 97 == 5:
            out += ["", "#comment 1 2 3"]
    end = "\r\n" if crlf else "\n"
    path.write_bytes((end.join(out) + end).encode())


def test_reader_matches_loadtxt_on_reference_catalogue():
    path = GOLDEN / "test_data_catalogue.txt"
    ref = np.loadtxt(path)
    cat = DeviceCatalogue.read_from_file(path, names=['x', 'y', 'z', 'nz'])
    assert cat.ntotal == 3
    for i, f in enumerate(['x', 'y', 'z', 'nz']):
        assert np.array_equal(cat[f], ref[:, i]), f
    assert np.array_equal(cat['w'], np.ones(3))
    assert cat.bounds == ParticleCatalogue(*ref.T).bounds


def test_reader_matches_loadtxt_and_oracle_bit_for_bit(tmp_path):
    rng = np.random.default_rng(11)
    a = np.column_stack([np.arange(20000), rng.uniform(-1e3, 1e3, (20000, 3)),
                         rng.uniform(0.5, 2., 20000)])
    a[7, 1] = -0.0
    a[8, 2] = 1e-310   # subnormal
    b = np.column_stack([np.arange(777), rng.normal(0., 300., (777, 3)),
                         rng.uniform(0.5, 2., 777)])
    pa, pb = tmp_path / "a.txt", tmp_path / "b.dat"
    _write(pa, a, seed=1)
    _write(pb, b, seed=2, crlf=True)
    names = ['id', 'z', 'x', 'y', 'wc']
    path = f"{pa}::{pb}"
    cat = DeviceCatalogue.read_from_file(path, names=names, volume=2.e9)
    ref = O.load_catalogue_text(path, ','.join(names), volume=2.e9)
    both = np.concatenate([np.loadtxt(pa), np.loadtxt(pb)])
    assert cat.ntotal == len(both)
    for f in ['x', 'y', 'z', 'nz', 'ws', 'wc', 'w']:
        assert np.array_equal(cat[f], ref[f]), f
        assert np.array_equal(np.signbit(cat[f]), np.signbit(ref[f])), f
    assert np.array_equal(cat['z'], both[:, 1])
    assert np.array_equal(cat['x'], both[:, 2])
    assert np.array_equal(cat['nz'], np.full(len(both), len(both) / 2.e9))
    assert cat.wtotal == pytest.approx(float(np.sum(ref['w'])), rel=1e-13)
    assert cat.wstotal == float(len(both))


def test_reader_errors_and_empty_files(tmp_path):
    p = tmp_path / "short.txt"
    p.write_text("1 2 3\n4 5\n")
    with pytest.raises(_lib.InvalidDataError, match="fewer than 3"):
        DeviceCatalogue.read_from_file(p, names=['x', 'y', 'z'])
    with pytest.raises(_lib.InvalidDataError, match="Failed to open"):
        DeviceCatalogue.read_from_file(tmp_path / "none.txt",
                                       names=['x', 'y', 'z'])
    with pytest.raises(_lib.InvalidDataError, match="HDF5"):
        DeviceCatalogue.read_from_file(tmp_path / "cat.hdf5",
                                       names=['x', 'y', 'z'])
    with pytest.raises(_lib.InvalidParameterError, match="'x', 'y' and 'z'"):
        DeviceCatalogue.read_from_file(p, names=['x', 'y'])
    e = tmp_path / "empty.txt"
    e.write_text("# nothing\n\n")
    cat = DeviceCatalogue.read_from_file(e, names=['x', 'y', 'z'])
    assert cat.ntotal == 0 and cat.wtotal == 0.
    assert cat.bounds == {ax: (0., 0.) for ax in 'xyz'}
    cat.periodise([100.] * 3)
    assert len(np.asarray(cat.compute_los())) == 0


def _pair(seed, n=50000, lo=-700., hi=900.):
    rng = np.random.default_rng(seed)
    d = rng.uniform(lo, hi, size=(n, 3))
    nz = rng.uniform(1e-4, 3e-4, n)
    ws, wc = rng.uniform(0.5, 1.5, (2, n))
    d[0] = 0.   # a particle at the origin: |x| = 0 line of sight
    host = ParticleCatalogue(*d.T, nz=nz, ws=ws, wc=wc)
    return host, DeviceCatalogue.from_catalogue(host)


def _same(host, dev):
    for f in ['x', 'y', 'z', 'nz', 'ws', 'wc']:
        assert np.array_equal(dev[f], host[f]), f
    assert dev.bounds == host.bounds


def test_device_preparation_is_bit_identical_to_host():
    box = [1200., 1500., 1800.]
    h, d = _pair(5)
    _same(h, d)
    assert np.array_equal(np.asarray(d.compute_los()), h.compute_los())
    assert d.wtotal == pytest.approx(h.wtotal, rel=1e-13)
    assert d.wstotal == pytest.approx(h.wstotal, rel=1e-13)
    for order in (2, 3):
        assert d._norm_sum(order) == pytest.approx(h._norm_sum(order),
                                                   rel=1e-13)
    assert d._has_nz() and h._has_nz()
    h.periodise(box)
    d.periodise(box)
    _same(h, d)
    # A pair: centring moves both by the randoms' mid-point.
    h2, d2 = _pair(6, n=20000, lo=-300., hi=500.)
    h.centre(box, catalogue_ref=h2)
    d.centre(box, catalogue_ref=d2)
    _same(h, d)
    _same(h2, d2)
    h.pad(box, boxsize_pad=[0.02, 0.03, 0.05], catalogue_ref=h2)
    d.pad(box, boxsize_pad=[0.02, 0.03, 0.05], catalogue_ref=d2)
    _same(h, d)
    _same(h2, d2)
    h.pad(box, ngrid=[64, 96, 80], ngrid_pad=[3., 2., 5.])
    d.pad(box, ngrid=[64, 96, 80], ngrid_pad=[3., 2., 5.])
    _same(h, d)
    h.compute_mean_density(boxsize=box)
    d.compute_mean_density(boxsize=box)
    _same(h, d)
    d['nz'] = 0.
    assert not d._has_nz()


def _raw(cat):
    return cat._libh, cat._ctx.handle, cat._h


def test_cabi_box_preparation_matches_cpp_restatements():
    h, d = _pair(9)
    lib, ctx, hd = _raw(d)
    box = [1000., 1100., 1300.]
    x, y, z = h['x'], h['y'], h['z']
    B = (C.c_double * 3)(*box)
    # pad_grids: ngrid_pad * boxsize / ngrid, left to right.
    ng, npad = (C.c_double * 3)(64., 96., 80.), (C.c_double * 3)(3., 2., 5.)
    _lib.check(lib.trvg_dcat_pad(ctx, hd, None, B, None, ng, npad))
    (px, py, pz), _ = O.pad_cpp(x, y, z, box, ngrid=[64, 96, 80],
                                ngrid_pad=[3., 2., 5.])
    assert np.array_equal(d['x'], px) and np.array_equal(d['y'], py)
    assert np.array_equal(d['z'], pz)
    # centre_in_box.
    _lib.check(lib.trvg_dcat_centre(ctx, hd, None, B))
    (cx, cy, cz), _ = O.centre(px, py, pz, box)
    assert np.array_equal(d['x'], cx) and np.array_equal(d['z'], cz)
    # offset_coords_for_periodicity on coordinates beyond both ends.
    _lib.check(lib.trvg_dcat_offset(ctx, hd, (C.c_double * 3)(
        -400., 900., 250.)))
    sx, sy, sz = cx + 400., cy - 900., cz - 250.
    _lib.check(lib.trvg_dcat_wrap_box(ctx, hd, B))
    wx, wy, wz = O.offset_coords_for_periodicity(sx, sy, sz, box)
    for f, w in zip('xyz', (wx, wy, wz)):
        assert np.array_equal(d[f], w), f


@pytest.mark.parametrize("precision", ['fp64', 'fp32mixed'])
def test_estimators_on_device_catalogues_match_goldens(
        precision, tmp_path, rand_catalogue_array):
    """The reference's golden measurements from catalogues read from text
    files straight into device memory."""
    rpath = tmp_path / "rand.txt"
    np.savetxt(rpath, rand_catalogue_array, fmt='%.17g')
    dpath = GOLDEN / "test_data_catalogue.txt"
    names = ['x', 'y', 'z', 'nz']
    bins = Binning('fourier', 'lin', *KBINS)
    samp = _sampling(precision)

    def dev():
        return (DeviceCatalogue.read_from_file(dpath, names=names),
                DeviceCatalogue.read_from_file(rpath, names=names))
    d, r = dev()
    ctx = d._ctx
    res = compute_bispec(d, r, degrees=(0, 0, 0), binning=bins, form='diag',
                         sampling_params=samp)
    assert ctx.stats()['h2d_bytes'] == 0
    _check_golden(res, load_golden('bk000_diag_lpp.txt'), 'bispec',
                  precision)
    d, r = dev()
    res = compute_bispec_in_gpp_box(d, degrees=(2, 0, 2), binning=bins,
                                    form='diag', sampling_params=samp)
    _check_golden(res, load_golden('bk202_diag_gpp.txt'), 'bispec',
                  precision)
    d, r = dev()
    res = compute_powspec(d, r, degree=2, binning=bins, sampling_params=samp)
    check_powspec(res, load_golden('pk2_lpp.txt'))


def test_device_and_host_catalogues_give_the_same_estimates(
        rand_catalogue_array):
    rng = np.random.default_rng(21)
    dd = rng.uniform(-500., 500., size=(4000, 3))
    r = rand_catalogue_array
    bins = Binning('fourier', 'lin', *KBINS)
    samp = _sampling('fp64')

    def host():
        return (ParticleCatalogue(*dd.T, nz=3e-9),
                ParticleCatalogue(r[:, 0], r[:, 1], r[:, 2], nz=r[:, 3]))
    hd, hr = host()
    ref = compute_bispec(hd, hr, degrees=(2, 0, 2), binning=bins,
                         form='full', sampling_params=samp)
    hd, hr = host()
    got = compute_bispec(DeviceCatalogue.from_catalogue(hd),
                         DeviceCatalogue.from_catalogue(hr),
                         degrees=(2, 0, 2), binning=bins, form='full',
                         sampling_params=samp)
    for k in ('bk_raw', 'bk_shot'):
        assert rel_err(got[k], ref[k]) < 1e-12, k
    # Explicit host lines of sight are uploaded.
    hd, hr = host()
    los = hd.compute_los() * 1.0
    got = compute_bispec(DeviceCatalogue.from_catalogue(hd),
                         DeviceCatalogue.from_catalogue(hr), los_data=los,
                         degrees=(2, 0, 2), binning=bins, form='full',
                         sampling_params=samp)
    assert rel_err(got['bk_raw'], ref['bk_raw']) < 1e-12


def test_batch_of_device_catalogues_matches_host_batch():
    box, sizes = 600., [1500, 4000, 2500]
    rng = np.random.default_rng(77)
    pos = [rng.uniform(0., box, size=(n, 3)) for n in sizes]
    binning = Binning('fourier', 'lin', 0.01, 0.1, 4)
    samp = _sampling('fp64', 32, box=box)
    kw = dict(degrees=(0, 0, 0), binning=binning, form='diag',
              sampling_params=samp)
    host = compute_bispec_in_gpp_box_batch(
        [ParticleCatalogue(*p.T, nz=len(p) / box ** 3) for p in pos], **kw)
    dev = compute_bispec_in_gpp_box_batch(
        [DeviceCatalogue(*p.T, nz=len(p) / box ** 3) for p in pos], **kw)
    for a, b in zip(dev, host):
        assert np.array_equal(a['nmodes_1'], b['nmodes_1'])
        for k in ('bk_raw', 'bk_shot'):
            assert rel_err(a[k], b[k]) < 1e-10, k


def test_device_catalogues_in_3pcf_window_and_powspec(rand_catalogue_array):
    """The 3PCF window (randoms alone), the periodic-box power spectrum and
    the survey 3PCF from device catalogues equal those from host ones."""
    from triumvirate_gb300.threept import compute_3pcf, compute_3pcf_window
    from triumvirate_gb300.twopt import compute_powspec_in_gpp_box
    r = rand_catalogue_array
    rng = np.random.default_rng(5)
    d = rng.uniform(-500., 500., size=(3000, 3))
    rb = Binning('config', 'lin', 50., 150., 4)
    kb = Binning('fourier', 'lin', *KBINS)
    samp = _sampling('fp64')

    def rc(device):
        cls = DeviceCatalogue if device else ParticleCatalogue
        return cls(r[:, 0], r[:, 1], r[:, 2], nz=r[:, 3])

    def dc(device):
        cls = DeviceCatalogue if device else ParticleCatalogue
        return cls(*d.T, nz=3e-9)
    for device in (False, True):
        w = compute_3pcf_window(rc(device), degrees=(2, 0, 2), binning=rb,
                                form='diag', sampling_params=samp)
        p = compute_powspec_in_gpp_box(dc(device), degree=2, binning=kb,
                                       sampling_params=samp)
        z = compute_3pcf(dc(device), rc(device), degrees=(0, 0, 0),
                         binning=rb, form='diag', sampling_params=samp)
        if not device:
            ref = (w, p, z)
    for got, want, keys in [(w, ref[0], ('zeta_raw', 'zeta_shot')),
                            (p, ref[1], ('pk_raw', 'pk_shot')),
                            (z, ref[2], ('zeta_raw', 'zeta_shot'))]:
        for k in keys:
            assert rel_err(got[k], want[k]) < 1e-12, k
