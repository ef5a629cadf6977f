"""Particle catalogues (mirrors ``triumvirate.catalogue.ParticleCatalogue``,
catalogue.py:55-865) with numpy columns instead of an astropy table."""
from __future__ import annotations

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

    # Arrays handed to the C ABI.
    def _columns(self):
        p = self._pdata
        w = np.ascontiguousarray(p['ws'] * p['wc'])
        return (np.ascontiguousarray(p['x']), np.ascontiguousarray(p['y']),
                np.ascontiguousarray(p['z']), w)
