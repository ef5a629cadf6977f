"""Marshalling between the Python API and the C ABI."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib

_SHAPE_OF_FORM = {'diag': 'diag', 'off-diag': 'off-diag', 'row': 'row',
                  'full': 'full', 'triu': 'triu'}


def make_params(paramset, npoint):
    """``trvg_params`` from a validated parameter dict."""
    p = _lib.Params()
    for i, ax in enumerate(['x', 'y', 'z']):
        p.boxsize[i] = float(paramset['boxsize'][ax])
        p.ngrid[i] = int(paramset['ngrid'][ax])
    p.assignment_order = int(paramset['assignment_order'])
    p.interlace = 0 if npoint == '3pt' else int(bool(paramset['interlace']))
    deg = paramset['degrees']
    p.ell1 = int(deg.get('ell1') or 0)
    p.ell2 = int(deg.get('ell2') or 0)
    p.ELL = int(deg.get('ELL') or 0)
    shape = paramset.get('shape') or paramset['form']
    p.shape = _lib.SHAPES[shape]
    p.idx_bin = int(paramset.get('idx_bin') or 0)
    p.precision = _lib.PRECISIONS[paramset.get('precision', 'fp64')]
    verbose = paramset.get('verbose', 0)
    p.verbose = int(verbose) if verbose is not None else 0
    wa = paramset.get('wa_orders') or {}
    p.i_wa = int(wa.get('i') or 0)
    p.j_wa = int(wa.get('j') or 0)
    return p


class HostBinning:
    """``trvg_binning`` over host arrays kept alive with the struct."""

    def __init__(self, binning):
        self.edges = np.ascontiguousarray(binning.bin_edges, dtype=np.float64)
        self.centres = np.ascontiguousarray(binning.bin_centres,
                                            dtype=np.float64)
        self.c = _lib.BinningC(int(binning.num_bins), _lib.dptr(self.edges),
                               _lib.dptr(self.centres))


class HostCatalogue:
    """``trvg_catalogue`` over host columns (and lines of sight)."""

    def __init__(self, x, y, z, w=None, los=None):
        self.cols = [np.ascontiguousarray(a, dtype=np.float64)
                     for a in (x, y, z)]
        self.w = None if w is None else np.ascontiguousarray(
            w, dtype=np.float64)
        self.los = None
        if los is not None:
            los = np.asarray(los, dtype=np.float64)
            self.los = [np.ascontiguousarray(los[:, i]) for i in range(3)]
        c = _lib.Catalogue()
        c.n = self.cols[0].shape[0]
        c.x, c.y, c.z = (a.ctypes.data for a in self.cols)
        c.w = None if self.w is None else self.w.ctypes.data
        if self.los is not None:
            c.los_x, c.los_y, c.los_z = (a.ctypes.data for a in self.los)
        c.memory = _lib.MEM_HOST
        self.c = c


def catalogue_arg(cat, los=None, with_los=False):
    """The ``trvg_catalogue`` (attribute ``c``) of a ParticleCatalogue
    (host columns) or a DeviceCatalogue (device columns, no copy), with
    lines of sight when `with_los` (`los`, else computed)."""
    if hasattr(cat, '_view'):
        return cat._view(los, with_los)
    x, y, z, w = cat._columns()
    if with_los and los is None:
        los = cat.compute_los()
    return HostCatalogue(x, y, z, w, np.asarray(los) if with_los else None)


def context_for(device, *catalogues):
    """The context of `device`; by default that of the first device
    catalogue among `catalogues`, else the process-wide default."""
    if device is None:
        for c in catalogues:
            if hasattr(c, '_ctx'):
                return c._ctx
    return _lib.default_context(device)


def device_catalogue(n, x_ptr, y_ptr, z_ptr, w_ptr=None, los_ptrs=None):
    """``trvg_catalogue`` over device pointers (e.g. torch ``data_ptr()``)."""
    c = _lib.Catalogue()
    c.n = int(n)
    c.x, c.y, c.z = int(x_ptr), int(y_ptr), int(z_ptr)
    c.w = None if w_ptr is None else int(w_ptr)
    if los_ptrs is not None:
        c.los_x, c.los_y, c.los_z = (int(p) for p in los_ptrs)
    c.memory = _lib.MEM_DEVICE
    return c


def dv_dim(shape, num_bins, idx_bin):
    d = C.c_int()
    _lib.check(_lib.load().trvg_data_vector_dim(
        _lib.SHAPES[shape], int(num_bins), int(idx_bin or 0), C.byref(d)))
    return d.value


class ThreeptResult:
    def __init__(self, dim):
        self.dim = dim
        self.c1b = np.zeros(dim)
        self.c1e = np.zeros(dim)
        self.n1 = np.zeros(dim, dtype=np.int32)
        self.c2b = np.zeros(dim)
        self.c2e = np.zeros(dim)
        self.n2 = np.zeros(dim, dtype=np.int32)
        self.raw = np.zeros(2 * dim)
        self.shot = np.zeros(2 * dim)
        self.c = _lib.ThreeptOut(
            dim, _lib.dptr(self.c1b), _lib.dptr(self.c1e), _lib.iptr(self.n1),
            _lib.dptr(self.c2b), _lib.dptr(self.c2e), _lib.iptr(self.n2),
            _lib.dptr(self.raw), _lib.dptr(self.shot))

    def as_dict(self, kind):
        raw = self.raw[0::2] + 1j * self.raw[1::2]
        shot = self.shot[0::2] + 1j * self.shot[1::2]
        if kind == 'bispec':
            return {'k1_bin': self.c1b, 'k1_eff': self.c1e,
                    'nmodes_1': self.n1.astype(np.int64),
                    'k2_bin': self.c2b, 'k2_eff': self.c2e,
                    'nmodes_2': self.n2.astype(np.int64),
                    'bk_raw': raw, 'bk_shot': shot}
        return {'r1_bin': self.c1b, 'r1_eff': self.c1e,
                'npairs_1': self.n1.astype(np.int64),
                'r2_bin': self.c2b, 'r2_eff': self.c2e,
                'npairs_2': self.n2.astype(np.int64),
                'zeta_raw': raw, 'zeta_shot': shot}


class PowspecResult:
    def __init__(self, dim):
        self.dim = dim
        self.kbin = np.zeros(dim)
        self.keff = np.zeros(dim)
        self.nmodes = np.zeros(dim, dtype=np.int32)
        self.raw = np.zeros(2 * dim)
        self.shot = np.zeros(2 * dim)
        self.c = _lib.PowspecOut(dim, _lib.dptr(self.kbin),
                                 _lib.dptr(self.keff), _lib.iptr(self.nmodes),
                                 _lib.dptr(self.raw), _lib.dptr(self.shot))

    def as_dict(self):
        return {'kbin': self.kbin, 'keff': self.keff,
                'nmodes': self.nmodes.astype(np.int64),
                'pk_raw': self.raw[0::2] + 1j * self.raw[1::2],
                'pk_shot': self.shot[0::2] + 1j * self.shot[1::2]}


def call_threept(fn_name, ctx, params, data_c, binning, norm, kind,
                 rand_c=None, alpha=None, shape=None, idx_bin=0):
    lib = _lib.load()
    dim = dv_dim(shape, binning.num_bins, idx_bin)
    res = ThreeptResult(dim)
    hb = HostBinning(binning)
    fn = getattr(lib, fn_name)
    if rand_c is None:
        st = fn(ctx.handle, C.byref(params), C.byref(data_c), C.byref(hb.c),
                float(norm), C.byref(res.c))
    else:
        st = fn(ctx.handle, C.byref(params), C.byref(data_c),
                C.byref(rand_c), float(alpha), C.byref(hb.c), float(norm),
                C.byref(res.c))
    _lib.check(st)
    return res.as_dict(kind)


def call_3pcf_window(ctx, params, rand_c, binning, norm, alpha, wide_angle,
                     shape=None, idx_bin=0):
    """trvg_compute_3pcf_window; the 3PCF result dictionary."""
    lib = _lib.load()
    res = ThreeptResult(dv_dim(shape, binning.num_bins, idx_bin))
    hb = HostBinning(binning)
    _lib.check(lib.trvg_compute_3pcf_window(
        ctx.handle, C.byref(params), C.byref(rand_c), float(alpha),
        C.byref(hb.c), float(norm), int(bool(wide_angle)), C.byref(res.c)))
    return res.as_dict('3pcf')


def call_bispec_batch(ctx, params, cat_c, offsets, binning, norms, shape,
                      idx_bin=0):
    """trvg_compute_bispec_in_gpp_box_batch over the concatenated catalogue
    `cat_c`; one result dictionary per mock."""
    lib = _lib.load()
    n_mocks = len(norms)
    dim = dv_dim(shape, binning.num_bins, idx_bin)
    res = [ThreeptResult(dim) for _ in range(n_mocks)]
    outs = (_lib.ThreeptOut * n_mocks)(*[r.c for r in res])
    off = np.ascontiguousarray(offsets, dtype=np.int64)
    nrm = np.ascontiguousarray(norms, dtype=np.float64)
    hb = HostBinning(binning)
    _lib.check(lib.trvg_compute_bispec_in_gpp_box_batch(
        ctx.handle, C.byref(params), C.byref(cat_c), int(n_mocks),
        off.ctypes.data_as(C.POINTER(C.c_int64)), C.byref(hb.c),
        _lib.dptr(nrm), outs))
    return [r.as_dict('bispec') for r in res]


def call_powspec(fn_name, ctx, params, data_c, binning, norm, rand_c=None,
                 alpha=None):
    lib = _lib.load()
    res = PowspecResult(int(binning.num_bins))
    hb = HostBinning(binning)
    fn = getattr(lib, fn_name)
    if rand_c is None:
        st = fn(ctx.handle, C.byref(params), C.byref(data_c), C.byref(hb.c),
                float(norm), C.byref(res.c))
    else:
        st = fn(ctx.handle, C.byref(params), C.byref(data_c),
                C.byref(rand_c), float(alpha), C.byref(hb.c), float(norm),
                C.byref(res.c))
    _lib.check(st)
    return res.as_dict()


def grid_powlaw_norm(ctx, params, cat_c, order):
    out = C.c_double()
    _lib.check(_lib.load().trvg_calc_grid_based_powlaw_norm(
        ctx.handle, C.byref(params), C.byref(cat_c), int(order),
        C.byref(out)))
    return out.value


def assign_mesh(ctx, params, cat_c, shadow=False):
    n = params.ngrid[0] * params.ngrid[1] * params.ngrid[2]
    mesh = np.zeros(n)
    _lib.check(_lib.load().trvg_assign_weighted_field_to_mesh(
        ctx.handle, C.byref(params), C.byref(cat_c), int(bool(shadow)),
        _lib.dptr(mesh)))
    return mesh.reshape(tuple(params.ngrid))
