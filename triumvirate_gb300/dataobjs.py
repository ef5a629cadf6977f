"""Binning (mirrors ``triumvirate.dataobjs.Binning``, dataobjs.pyx:16-224,
and ``trv::Binning``, dataobjs.cpp:39-266)."""
from __future__ import annotations

import math

import numpy as np


class Binning:
    """Binning of a coordinate space.

    Parameters
    ----------
    space : {'config', 'fourier'}
        Coordinate space.
    scheme : {'lin', 'log', 'linpad', 'logpad'}
        Binning scheme (linear or logarithmic, optionally padded from zero
        by 5 linear bins).
    bin_min, bin_max : float, optional
        Bin range.
    num_bins : int, optional
        Number of bins.
    """

    NBIN_PAD = 5                 # dataobjs.hpp:144
    DBIN_PAD_FOURIER = 1.e-3     # dataobjs.hpp:145
    DBIN_PAD_CONFIG = 10.        # dataobjs.hpp:146

    def __init__(self, space, scheme, bin_min=None, bin_max=None,
                 num_bins=None):
        if space not in ('config', 'fourier'):
            raise ValueError(f"Unrecognised coordinate space: {space}.")
        self.space = space
        self.scheme = scheme
        self.bin_min = bin_min
        self.bin_max = bin_max
        self.num_bins = num_bins
        self._dbin_pad = (self.DBIN_PAD_FOURIER if space == 'fourier'
                          else self.DBIN_PAD_CONFIG)
        self.bin_edges, self.bin_centres, self.bin_widths = [], [], []
        if None not in (bin_min, bin_max, num_bins):
            self.set_bins(bin_min, bin_max, num_bins)

    @classmethod
    def from_parameter_set(cls, paramset):
        """Binning from a parameter set (dataobjs.pyx:96-133)."""
        if paramset['space'] not in ['fourier', 'config']:
            raise ValueError(
                "'space' parameter is unset or unrecognised in `paramset`.")
        return cls(paramset['space'], paramset['binning'],
                   bin_min=paramset['range'][0],
                   bin_max=paramset['range'][-1],
                   num_bins=paramset['num_bins'])

    def set_bins(self, bin_min, bin_max, num_bins):
        """Bins from a range and number (dataobjs.cpp:56-72, 134-221)."""
        if bin_min < 0.:
            raise ValueError("Bin range must be non-negative.")
        if num_bins <= 0:
            raise ValueError("Number of bins must be positive.")
        self.bin_min = float(bin_min)
        self.bin_max = float(bin_max)
        self.num_bins = int(num_bins)
        self._compute()

    def set_grid_based_bins(self, boxsize, ngrid=None):
        """Linear bins at the grid resolution (dataobjs.cpp:81-107)."""
        boxsize_max = max(np.atleast_1d(boxsize))
        ngrid_min = min(np.atleast_1d(ngrid))
        self.scheme = 'lin'
        self.bin_min = 0.
        if self.space == 'config':
            width = boxsize_max / float(ngrid_min)
            self.bin_max = boxsize_max / 2.
        else:
            width = 2 * math.pi / boxsize_max
            self.bin_max = math.pi * float(ngrid_min) / boxsize_max
        self.bin_max += width / 2.
        self.num_bins = int(ngrid_min) // 2
        self._compute()

    def set_bins_from_edges(self, bin_edges):
        """Custom bins from edges (dataobjs.cpp:109-132)."""
        edges = [float(e) for e in bin_edges]
        self.bin_min, self.bin_max = edges[0], edges[-1]
        self.num_bins = len(edges) - 1
        self.scheme = 'custom'
        self.bin_edges = edges
        self.bin_centres = [(edges[i] + edges[i + 1]) / 2.
                            for i in range(self.num_bins)]
        self.bin_widths = [edges[i + 1] - edges[i]
                           for i in range(self.num_bins)]

    def _compute(self):
        edges, centres, widths = [], [], []
        nb, lo, hi = self.num_bins, self.bin_min, self.bin_max
        pad, npad = self._dbin_pad, self.NBIN_PAD
        if self.scheme == 'lin':
            dbin = (hi - lo) / float(nb)
            for i in range(nb):
                left = lo + dbin * i
                edges.append(left)
                centres.append(left + dbin / 2.)
                widths.append(dbin)
            edges.append(hi)
        elif self.scheme == 'log':
            if lo == 0.:
                raise ValueError("Cannot use logarithmic binning when the "
                                 "lowest edge is zero.")
            dln = (math.log(hi) - math.log(lo)) / float(nb)
            for i in range(nb):
                left = lo * math.exp(dln * i)
                right = lo * math.exp(dln * (i + 1))
                edges.append(left)
                centres.append((left + right) / 2.)
                widths.append(right - left)
            edges.append(hi)
        elif self.scheme in ('linpad', 'logpad'):
            for i in range(npad):
                left = pad * i
                edges.append(left)
                centres.append(left + pad / 2.)
                widths.append(pad)
            start = pad * npad
            if self.scheme == 'linpad':
                dbin = (hi - start) / float(nb - npad)
                for i in range(npad, nb):
                    left = start + dbin * (i - npad)
                    edges.append(left)
                    centres.append(left + dbin / 2.)
                    widths.append(dbin)
            else:
                dln = (math.log(hi) - math.log(start)) / float(nb - npad)
                for i in range(npad, nb):
                    left = start * math.exp(dln * (i - npad))
                    right = start * math.exp(dln * (i - npad + 1))
                    edges.append(left)
                    centres.append((left + right) / 2.)
                    widths.append(right - left)
            edges.append(hi)
        else:
            raise ValueError(
                f"Unrecognised/unsupported binning `scheme`: {self.scheme}.")
        self.bin_edges, self.bin_centres, self.bin_widths = \
            edges, centres, widths

    def __repr__(self):
        return (f"Binning(space={self.space!r}, scheme={self.scheme!r}, "
                f"bin_min={self.bin_min}, bin_max={self.bin_max}, "
                f"num_bins={self.num_bins})")
