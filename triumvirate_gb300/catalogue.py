"""Particle catalogues (mirrors ``triumvirate.catalogue.ParticleCatalogue``,
catalogue.py:55-865): ``ParticleCatalogue`` holds numpy columns instead of
an astropy table; ``DeviceCatalogue`` holds the same columns in GPU memory,
read from files by the library's multi-threaded reader and prepared
(centred, padded, periodised, lines of sight) by device kernels."""
from __future__ import annotations

import ctypes as C
import warnings

import numpy as np


class ParticleCatalogue:
    """Particle catalogue with columns 'x', 'y', 'z', 'nz', 'ws', 'wc'.

    Parameters
    ----------
    x, y, z : array_like
        Cartesian coordinates.
    nz : array_like or float, optional
        Redshift-dependent mean number density (0 if `None`).
    ws, wc : array_like or float, optional
        Sample and clustering weights (default 1).  The overall weight of
        each particle is ``ws * wc``.
    logger : logging.Logger, optional
        Logger.
    """

    def __init__(self, x, y, z, nz=None, ws=1., wc=1., logger=None):
        self._logger = logger
        if nz is None:
            warnings.warn("Catalogue 'nz' field is None and thus set to "
                          "zero, which may raise errors in some "
                          "computations.")
            nz = 0.
        x = np.ascontiguousarray(x, dtype=np.float64)
        n = x.shape[0]

        def col(v):
            v = np.asarray(v, dtype=np.float64)
            return np.ascontiguousarray(np.broadcast_to(v, (n,)).copy()
                                        if v.ndim == 0 else v)

        self._pdata = {
            'x': x, 'y': col(y), 'z': col(z), 'nz': col(nz),
            'ws': col(ws), 'wc': col(wc),
        }
        self._source = f'extdata:{id(self._pdata)}'
        self._calc_bounds(init=True)
        self.ntotal = n
        self.wtotal = float(np.sum(self._pdata['ws'] * self._pdata['wc']))
        self.wstotal = float(np.sum(self._pdata['ws']))
        if logger:
            logger.info("Catalogue initialised: ntotal = %d, wtotal = %.3f, "
                        "wstotal = %.3f.", self.ntotal, self.wtotal,
                        self.wstotal)

    @classmethod
    def read_from_file(cls, filepath, names=None, logger=None, **kwargs):
        """Read a plain-text catalogue with columns `names`."""
        data = np.loadtxt(filepath, ndmin=2)
        names = names or ['x', 'y', 'z', 'nz', 'ws', 'wc'][:data.shape[1]]
        cols = {nm: data[:, i] for i, nm in enumerate(names)}
        cat = cls(cols['x'], cols['y'], cols['z'], nz=cols.get('nz'),
                  ws=cols.get('ws', 1.), wc=cols.get('wc', 1.),
                  logger=logger)
        cat._source = f'extfile:{filepath}'
        return cat

    def __len__(self):
        return self.ntotal

    def __str__(self):
        return f"ParticleCatalogue({self._source})"

    def __getitem__(self, key):
        if isinstance(key, str):
            return self._pdata[key]
        return {k: v[key] for k, v in self._pdata.items()}

    def __setitem__(self, key, val):
        if not isinstance(key, str):
            raise ValueError('Cannot set values for non-string-type key.')
        self._pdata[key] = np.ascontiguousarray(
            np.broadcast_to(np.asarray(val, dtype=np.float64),
                            (self.ntotal,)).copy())

    @property
    def bounds(self):
        return self._bounds

    def _calc_bounds(self, init=False):
        self._bounds = {ax: (float(np.min(self._pdata[ax])),
                             float(np.max(self._pdata[ax])))
                        if self._pdata[ax].size else (0., 0.)
                        for ax in ('x', 'y', 'z')}

    def _check_bounds_in_boxsize(self, boxsize):
        return [ax for iax, ax in enumerate(['x', 'y', 'z'])
                if self._bounds[ax][1] - self._bounds[ax][0] > boxsize[iax]]

    def compute_los(self):
        """Unit end-point lines of sight (catalogue.py:437-458)."""
        x, y, z = self._pdata['x'], self._pdata['y'], self._pdata['z']
        n = np.sqrt(x ** 2 + y ** 2 + z ** 2)
        n[n == 0.] = 1.
        return np.transpose([x / n, y / n, z / n])

    def compute_mean_density(self, volume=None, boxsize=None):
        """Set 'nz' to ntotal / volume (catalogue.py:460-488)."""
        if np.isscalar(boxsize):
            boxsize = [boxsize] * 3
        volume = volume or np.prod(boxsize)
        self['nz'] = self.ntotal / volume

    def offset_coords(self, origin):
        for axis, coord in zip(['x', 'y', 'z'], origin):
            self._pdata[axis] = self._pdata[axis] - coord
        self._calc_bounds()

    def centre(self, boxsize, catalogue_ref=None):
        """Centre (a pair of) catalogues in a box (catalogue.py:490-545)."""
        if np.isscalar(boxsize):
            boxsize = [boxsize] * 3
        ref = self if catalogue_ref is None else catalogue_ref
        if self._check_bounds_in_boxsize(boxsize):
            warnings.warn("Catalogue extent exceeds the box size.")
        origin = np.array([np.mean(ref.bounds[ax]) - boxsize[i] / 2.
                           for i, ax in enumerate(['x', 'y', 'z'])])
        self.offset_coords(origin)
        if catalogue_ref is not None:
            catalogue_ref.offset_coords(origin)

    def pad(self, boxsize, ngrid=None, boxsize_pad=None, ngrid_pad=None,
            catalogue_ref=None):
        """Pad (a pair of) catalogues in a box (catalogue.py:547-646)."""
        if boxsize_pad is None and ngrid_pad is None:
            warnings.warn("`boxsize_pad` and `ngrid_pad` are both None. "
                          "No padding is applied to the catalogue.")
            return
        if boxsize_pad is not None and ngrid_pad is not None:
            raise ValueError("Conflicting padding as `boxsize_pad` and "
                             "`ngrid_pad` are both set (not None).")
        if np.isscalar(boxsize):
            boxsize = [boxsize] * 3
        ref = self if catalogue_ref is None else catalogue_ref
        origin = np.array([ref.bounds[ax][0] for ax in ['x', 'y', 'z']])
        if boxsize_pad:
            origin -= np.multiply(boxsize_pad, boxsize)
        if ngrid_pad:
            origin -= np.multiply(ngrid_pad, np.divide(boxsize, ngrid))
        self.offset_coords(origin)
        if catalogue_ref is not None:
            catalogue_ref.offset_coords(origin)

    def periodise(self, boxsize):
        """Centre and wrap into a periodic box (catalogue.py:648-676)."""
        if np.isscalar(boxsize):
            boxsize = [boxsize] * 3
        if self._check_bounds_in_boxsize(boxsize):
            warnings.warn("Box size is smaller than particle coordinate "
                          "extents.")
        for i, ax in enumerate(['x', 'y', 'z']):
            lo, hi = self._bounds[ax]
            self._pdata[ax] = (self._pdata[ax] + boxsize[i] / 2.
                               - (hi + lo) / 2.) % boxsize[i]
        self._calc_bounds()

    def write_attrs_as_header(self, catalogue_ref=None):
        """Catalogue attributes as a measurement-file header
        (catalogue.py:803-858 of the library)."""
        def one(cat, name, extents):
            b = cat.bounds
            return "\n".join([
                f"{name} source: {cat._source}",
                f"{name} size: ntotal = {cat.ntotal:d}, "
                f"wtotal = {cat.wtotal:.3f}, wstotal = {cat.wstotal:.3f}",
                f"{extents} particle extents: "
                f"([{b['x'][0]:.3f}, {b['x'][1]:.3f}], "
                f"[{b['y'][0]:.3f}, {b['y'][1]:.3f}], "
                f"[{b['z'][0]:.3f}, {b['z'][1]:.3f}])",
            ])
        if catalogue_ref is None:
            return one(self, "Catalogue", "Catalogue")
        return "\n".join([one(self, "Data catalogue", "Data-source"),
                          one(catalogue_ref, "Random catalogue",
                              "Random-source")])

    # Sums behind the particle normalisation and the 'nz' check.
    def _norm_sum(self, order):
        p = self._pdata
        if order == 3:
            return float(np.sum(p['ws'] * p['nz'] ** 2 * p['wc'] ** 3))
        return float(np.sum(p['ws'] * p['nz'] * p['wc'] ** 2))

    def _has_nz(self):
        return bool(self._pdata['nz'].any())

    # Arrays handed to the C ABI.
    def _columns(self):
        p = self._pdata
        w = np.ascontiguousarray(p['ws'] * p['wc'])
        return (np.ascontiguousarray(p['x']), np.ascontiguousarray(p['y']),
                np.ascontiguousarray(p['z']), w)


_FIELDS = ['x', 'y', 'z', 'nz', 'ws', 'wc']


def _triple(v):
    return [float(v)] * 3 if np.isscalar(v) else [float(a) for a in v]


def _dvec(v):
    return (C.c_double * 3)(*_triple(v))


class DeviceLOS:
    """Lines of sight of a ``DeviceCatalogue``, kept in device memory; an
    (N, 3) host array on demand (``np.asarray``)."""

    def __init__(self, catalogue):
        self._cat = catalogue

    @property
    def shape(self):
        return (self._cat.ntotal, 3)

    def __len__(self):
        return self._cat.ntotal

    def __array__(self, dtype=None, copy=None):
        a = np.stack([self._cat[f'los_{ax}'] for ax in 'xyz'], axis=1)
        return a if dtype is None else a.astype(dtype)


class DeviceCatalogue:
    """Particle catalogue held in GPU memory.

    Same interface as ``ParticleCatalogue`` (indexing by column, `bounds`,
    `ntotal`, `wtotal`, `wstotal`, `compute_los`, `compute_mean_density`,
    `offset_coords`, `centre`, `pad`, `periodise`), and accepted by every
    estimator in place of one; the coordinates never leave the device.
    Coordinate transforms give the same bits as ``ParticleCatalogue``; the
    weight totals come from a fixed-order device reduction.

    Parameters
    ----------
    x, y, z, nz, ws, wc, logger :
        As for ``ParticleCatalogue``.
    device : int, optional
        CUDA device (default: the process-wide default context's).
    """

    def __init__(self, x, y, z, nz=None, ws=1., wc=1., logger=None,
                 device=None):
        if nz is None:
            warnings.warn("Catalogue 'nz' field is None and thus set to "
                          "zero, which may raise errors in some "
                          "computations.")
            nz = 0.
        x = np.ascontiguousarray(x, dtype=np.float64)
        n = x.shape[0]

        def col(v):
            v = np.asarray(v, dtype=np.float64)
            return np.ascontiguousarray(np.broadcast_to(v, (n,)))

        cols = [x, col(y), col(z), col(nz), col(ws), col(wc)]
        from . import _lib
        self._init(device, logger)
        h = C.c_void_p()
        _lib.check(self._libh.trvg_dcat_from_host(
            self._ctx.handle, n, *(_lib.dptr(c) for c in cols), C.byref(h)))
        self._finish(h, f'extdata:{id(self)}')

    def _init(self, device, logger):
        from . import _lib
        self._libh = _lib.load()
        self._ctx = _lib.default_context(device)
        self.device = self._ctx.device
        self._logger = logger
        self._h = None

    def _finish(self, handle, source):
        self._h = handle
        self._source = source
        self._los = None
        self._totals = None
        self._calc_bounds()
        n = C.c_int64()
        self._call('trvg_dcat_info', C.byref(n), None, None, None, None)
        self.ntotal = int(n.value)
        if self._logger:
            self._logger.info(
                "Catalogue initialised on the device: ntotal = %d, "
                "wtotal = %.3f, wstotal = %.3f.", self.ntotal, self.wtotal,
                self.wstotal)

    def _call(self, fn, *args):
        from . import _lib
        _lib.check(getattr(self._libh, fn)(self._ctx.handle, self._h, *args))

    @classmethod
    def read_from_file(cls, filepath, names=None, volume=0., logger=None,
                       device=None):
        """Read a plain-text catalogue (``load_catalogue_file``,
        particles.cpp:94-510): columns `names` (default: x, y, z, nz, ws,
        wc, as many as the first data row has), sub-files joined by "::";
        absent 'nz' becomes ntotal / `volume` (0 if `volume` <= 0), absent
        weights 1."""
        if names is None:
            first = str(filepath).split('::')[0]
            ncol = 0
            with open(first) as f:
                for line in f:
                    if line.strip() and not line.startswith('#'):
                        ncol = len(line.split())
                        break
            names = _FIELDS[:max(ncol, 3)]
        from . import _lib
        cat = cls.__new__(cls)
        cat._init(device, logger)
        h = C.c_void_p()
        _lib.check(cat._libh.trvg_dcat_read_text(
            cat._ctx.handle, str(filepath).encode(),
            ','.join(names).encode(), float(volume or 0.), C.byref(h)))
        cat._finish(h, f'extfile:{filepath}')
        return cat

    @classmethod
    def from_catalogue(cls, catalogue, device=None):
        """Copy a ``ParticleCatalogue`` to the device."""
        cat = cls(catalogue['x'], catalogue['y'], catalogue['z'],
                  nz=catalogue['nz'], ws=catalogue['ws'], wc=catalogue['wc'],
                  logger=getattr(catalogue, '_logger', None), device=device)
        cat._source = catalogue._source
        return cat

    @classmethod
    def concatenate(cls, catalogues, device=None):
        """One device catalogue holding `catalogues` back to back (device
        copies; host catalogues are uploaded first)."""
        from . import _lib
        parts = [c if isinstance(c, DeviceCatalogue)
                 else DeviceCatalogue.from_catalogue(c, device=device)
                 for c in catalogues]
        cat = cls.__new__(cls)
        cat._init(parts[0].device if parts and device is None else device,
                  None)
        arr = (C.c_void_p * max(len(parts), 1))(*(p._h.value for p in parts))
        h = C.c_void_p()
        _lib.check(cat._libh.trvg_dcat_concat(cat._ctx.handle, arr,
                                              len(parts), C.byref(h)))
        cat._finish(h, 'concatenated')
        return cat

    def __del__(self):
        h = getattr(self, '_h', None)
        if h is not None and h.value:
            try:
                self._libh.trvg_dcat_destroy(h)
            except Exception:  # interpreter shutting down
                pass
            self._h = None

    def __len__(self):
        return self.ntotal

    def __str__(self):
        return f"DeviceCatalogue({self._source})"

    def __getitem__(self, key):
        if not isinstance(key, str):
            raise ValueError('Device catalogues are indexed by column name.')
        out = np.empty(self.ntotal)
        from . import _lib
        self._call('trvg_dcat_download', key.encode(), _lib.dptr(out))
        return out

    def __setitem__(self, key, val):
        if not isinstance(key, str):
            raise ValueError('Cannot set values for non-string-type key.')
        from . import _lib
        if np.ndim(val) == 0 and key in ('nz', 'ws', 'wc'):
            self._call('trvg_dcat_set_column', key.encode(), float(val))
        else:
            a = np.ascontiguousarray(np.broadcast_to(
                np.asarray(val, dtype=np.float64), (self.ntotal,)))
            self._call('trvg_dcat_upload', key.encode(), _lib.dptr(a))
        if key in ('x', 'y', 'z'):
            self._calc_bounds()
        if key in ('ws', 'wc'):
            self._totals = None

    @property
    def wtotal(self):
        return self._weight_totals()[0]

    @property
    def wstotal(self):
        return self._weight_totals()[1]

    def _weight_totals(self):
        if self._totals is None:
            w, ws = C.c_double(), C.c_double()
            self._call('trvg_dcat_info', None, C.byref(w), C.byref(ws),
                       None, None)
            self._totals = (w.value, ws.value)
        return self._totals

    @property
    def bounds(self):
        return self._bounds

    def _calc_bounds(self):
        lo, hi = (C.c_double * 3)(), (C.c_double * 3)()
        self._call('trvg_dcat_info', None, None, None, lo, hi)
        self._bounds = {ax: (float(lo[i]), float(hi[i]))
                        for i, ax in enumerate(['x', 'y', 'z'])}

    def _check_bounds_in_boxsize(self, boxsize):
        return [ax for iax, ax in enumerate(['x', 'y', 'z'])
                if self._bounds[ax][1] - self._bounds[ax][0] > boxsize[iax]]

    def compute_los(self):
        """Unit end-point lines of sight, computed and kept on the device
        (catalogue.py:437-458)."""
        self._call('trvg_dcat_compute_los')
        self._los = DeviceLOS(self)
        return self._los

    def compute_mean_density(self, volume=None, boxsize=None):
        """Set 'nz' to ntotal / volume (catalogue.py:460-488)."""
        if np.isscalar(boxsize):
            boxsize = [boxsize] * 3
        volume = volume or np.prod(boxsize)
        self['nz'] = self.ntotal / volume

    def offset_coords(self, origin):
        self._call('trvg_dcat_offset', _dvec(origin))
        self._calc_bounds()

    def centre(self, boxsize, catalogue_ref=None):
        """Centre (a pair of) catalogues in a box (catalogue.py:490-545)."""
        if np.isscalar(boxsize):
            boxsize = [boxsize] * 3
        ref = self if catalogue_ref is None else catalogue_ref
        if self._check_bounds_in_boxsize(boxsize):
            warnings.warn("Catalogue extent exceeds the box size.")
        origin = np.array([np.mean(ref.bounds[ax]) - boxsize[i] / 2.
                           for i, ax in enumerate(['x', 'y', 'z'])])
        self.offset_coords(origin)
        if catalogue_ref is not None:
            catalogue_ref.offset_coords(origin)

    def pad(self, boxsize, ngrid=None, boxsize_pad=None, ngrid_pad=None,
            catalogue_ref=None):
        """Pad (a pair of) catalogues in a box (catalogue.py:547-646)."""
        if boxsize_pad is None and ngrid_pad is None:
            warnings.warn("`boxsize_pad` and `ngrid_pad` are both None. "
                          "No padding is applied to the catalogue.")
            return
        if boxsize_pad is not None and ngrid_pad is not None:
            raise ValueError("Conflicting padding as `boxsize_pad` and "
                             "`ngrid_pad` are both set (not None).")
        if np.isscalar(boxsize):
            boxsize = [boxsize] * 3
        ref = self if catalogue_ref is None else catalogue_ref
        origin = np.array([ref.bounds[ax][0] for ax in ['x', 'y', 'z']])
        if boxsize_pad:
            origin -= np.multiply(boxsize_pad, boxsize)
        if ngrid_pad:
            origin -= np.multiply(ngrid_pad, np.divide(boxsize, ngrid))
        self.offset_coords(origin)
        if catalogue_ref is not None:
            catalogue_ref.offset_coords(origin)

    def periodise(self, boxsize):
        """Centre and wrap into a periodic box on the device
        (catalogue.py:648-676)."""
        if np.isscalar(boxsize):
            boxsize = [boxsize] * 3
        if self._check_bounds_in_boxsize(boxsize):
            warnings.warn("Box size is smaller than particle coordinate "
                          "extents.")
        self._call('trvg_dcat_periodise', _dvec(boxsize))
        self._calc_bounds()

    def wrap_box(self, boxsize):
        """Fold coordinates into [0, L) as the C++ programs do
        (``offset_coords_for_periodicity``, particles.cpp:678-699)."""
        self._call('trvg_dcat_wrap_box', _dvec(boxsize))
        self._calc_bounds()

    write_attrs_as_header = ParticleCatalogue.write_attrs_as_header

    def _norm_sum(self, order):
        s = C.c_double()
        self._call('trvg_dcat_norm_sum', int(order), C.byref(s), None)
        return s.value

    def _has_nz(self):
        k = C.c_int64()
        self._call('trvg_dcat_norm_sum', 2, None, C.byref(k))
        return k.value > 0

    def _view(self, los=None, with_los=False):
        """``trvg_catalogue`` over the device columns (with lines of sight
        when `with_los`: `los` uploaded if given as host values, computed on
        the device if absent)."""
        from . import _lib
        if with_los:
            if los is None:
                if self._los is None:
                    self.compute_los()
            elif not (isinstance(los, DeviceLOS) and los._cat is self):
                a = np.asarray(los, dtype=np.float64)
                for i, ax in enumerate('xyz'):
                    self[f'los_{ax}'] = np.ascontiguousarray(a[:, i])
                self._los = DeviceLOS(self)
        c = _lib.Catalogue()
        _lib.check(self._libh.trvg_dcat_view(self._h, C.byref(c)))
        if not with_los:
            c.los_x = c.los_y = c.los_z = None
        return _View(c, self)


class _View:
    """Keeps the owning catalogue alive with its ``trvg_catalogue``."""

    def __init__(self, c, owner):
        self.c = c
        self._owner = owner
