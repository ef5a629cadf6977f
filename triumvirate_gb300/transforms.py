"""Spherical-Bessel transforms by FFTLog and log / linear resampling
(mirror of the reference's ``transforms.py``).

``SphericalBesselTransform`` turns a Hankel transform of order l + 1/2 into

    g(k) = int_0^inf r^2 dr (k r)^q j_l(k r) f(r)

with the factors r^{3/2} before and (2 pi / k)^{3/2} after (so that
``transform_cosmo_multipoles`` is 4 pi i^{-l} times the usual spherical
Bessel transform, and (2 pi)^-3 i^l times it backwards).
``DoubleSphericalBesselTransform`` applies one along each axis of a 2-d
array; every row (then every column) goes to the GPU in one batched call.
Extrapolation options 1-5 are supported ('outer' layer: the samples are
extended before the pre-factors, 'native': inside the FFTLog plan, options
1-4).
"""
from collections.abc import Sequence

import numpy as np
from scipy.interpolate import InterpolatedUnivariateSpline, RectBivariateSpline

from ._arrayops import (extrap2d_lin, extrap2d_loglin, extrap2d_loglin_oscil,
                        extrap2d_pad, extrap_lin, extrap_loglin,
                        extrap_loglin_oscil, extrap_pad)
from ._fftlog import HankelTransform


def _extend(arr, option, n_ext):
    if option == 1:
        return extrap_pad(arr, n_ext, 0., 0.)
    if option == 2:
        return extrap_pad(arr, n_ext, arr[0], arr[-1])
    if option == 3:
        return extrap_lin(arr, n_ext)
    if option == 4:
        return extrap_loglin(arr, n_ext)
    if option == 5:
        return extrap_loglin_oscil(arr, n_ext)
    return np.asarray(arr)


def _check_extrap(extrap, nsamp):
    if extrap not in {0, 1, 2, 3, 4, 5}:
        raise ValueError(f"Extrapolation option must be in 0 to 5: {extrap=}.")
    if extrap and nsamp % 2:
        raise ValueError("Input sample size must be even when extrapolation "
                         f"is used: {nsamp=}.")


def _cosmo_factors(direction, degree_sum):
    if direction in {'forward', 1}:
        return (-1j) ** degree_sum, 1.
    if direction in {'backward', -1}:
        return (1j) ** degree_sum, (2 * np.pi) ** (-3)
    raise ValueError(
        "Transform direction must be 'forward'/1 or 'backward'/-1.")


class SphericalBesselTransform:
    """Spherical Bessel transform of `degree` and power-law `bias` on the
    log-spaced `sample_pts` (reference transforms.py:35-272)."""

    def __init__(self, degree, bias, sample_pts, pivot=1., lowring=True,
                 extrap=0, extrap_exp=2., extrap_layer='outer',
                 threaded=False):
        sample_pts = np.asarray(sample_pts, dtype=float)
        _check_extrap(extrap, len(sample_pts))
        self.degree = degree
        self.bias = bias
        self._lowring = lowring
        self._extrap = extrap
        self._extrap_layer = extrap_layer
        native, self._n_ext = 0, 0
        if extrap:
            if extrap_layer == 'native':
                native = extrap
            elif extrap_layer == 'outer':
                nt = int(2 ** np.ceil(np.log2(extrap_exp * len(sample_pts))))
                self._n_ext = (nt - len(sample_pts)) // 2
                sample_pts = extrap_loglin(sample_pts, self._n_ext)
            else:
                raise ValueError("Extrapolation layer must be 'native' or "
                                 f"'outer': extrap_layer={extrap_layer}.")
        self._fbht = HankelTransform(degree + 0.5, bias, sample_pts,
                                     kr_c=pivot, lowring=lowring,
                                     extrap=native, extrap_exp=extrap_exp,
                                     threaded=threaded)
        self._post_slice = (slice(self._n_ext, -self._n_ext) if self._n_ext
                            else slice(None))
        self._logres = self._fbht._logres
        self._pre_sampts = np.asarray(self._fbht._pre_sampts)
        self._post_sampts = np.asarray(
            self._fbht._post_sampts)[self._post_slice]

    @property
    def size(self):
        """Sample size of the transform."""
        return self._fbht.size

    @property
    def pivot(self):
        """Pivot value."""
        return self._fbht._pivot

    def _perform_extrap(self, arr):
        return _extend(arr, self._extrap, self._n_ext)

    def _transform_rows(self, rows):
        """Transform the rows of a 2-d array of pre-transform samples (the
        'outer' extension included) in one batched call."""
        rows = np.asarray(rows) * self._pre_sampts ** 1.5
        _, out = self._fbht.transform(rows)
        out = out[..., self._post_slice]
        return out * (2 * np.pi / self._post_sampts) ** 1.5

    def transform(self, pre_samples):
        """Post-transform sample points and samples of 1-d `pre_samples`."""
        pre = np.asarray(pre_samples)
        if self._extrap_layer == 'outer':
            pre = self._perform_extrap(pre)
        out = self._transform_rows(pre[None, :])[0]
        return self._post_sampts.copy(), out

    def transform_cosmo_multipoles(self, direction, pre_samples):
        """Configuration <-> Fourier space multipoles ('forward'/1 from
        configuration space, 'backward'/-1 to it)."""
        parity, prefactor = _cosmo_factors(direction, self.degree)
        post_sampts, post_samples = self.transform(pre_samples)
        return post_sampts, post_samples * (prefactor * parity)


class DoubleSphericalBesselTransform:
    """Spherical Bessel transforms of `degrees` and `biases` along the two
    axes of a 2-d array (reference transforms.py:275-523)."""

    def __init__(self, degrees, biases, sample_pts, pivot=1., lowring=True,
                 extrap=0, extrap_exp=2., extrap2d=False, threaded=False):
        sample_pts = np.asarray(sample_pts, dtype=float)
        _check_extrap(extrap, len(sample_pts))
        self.degrees = degrees
        self.biases = biases
        self._lowring = lowring
        self._extrap = extrap
        self._extrap2d = extrap2d
        native, self._n_ext = 0, 0
        if extrap:
            if not extrap2d:
                native = extrap
            else:
                nt = int(2 ** np.ceil(np.log2(extrap_exp * len(sample_pts))))
                self._n_ext = (nt - len(sample_pts)) // 2
                sample_pts = extrap_loglin(sample_pts, self._n_ext)
        self._fbsjt = tuple(
            SphericalBesselTransform(d, b, sample_pts, pivot=pivot,
                                     lowring=lowring, extrap=native,
                                     extrap_exp=extrap_exp,
                                     threaded=threaded)
            for d, b in zip(degrees, biases))
        self._rep = 0
        self._post_slice = (slice(self._n_ext, -self._n_ext) if self._n_ext
                            else slice(None))
        self._logres = self._fbsjt[self._rep]._logres
        self._pre_sampts = np.asarray(self._fbsjt[self._rep]._pre_sampts)
        self._post_sampts = np.asarray(
            self._fbsjt[self._rep]._post_sampts)[self._post_slice]

    @property
    def size(self):
        """Sample size of the transform."""
        return self._fbsjt[self._rep].size

    @property
    def pivot(self):
        """Pivot values of the two axes."""
        return (self._fbsjt[0]._fbht._pivot, self._fbsjt[1]._fbht._pivot)

    def _perform_extrap(self, arr):
        if self._extrap == 1:
            return extrap2d_pad(arr, self._n_ext, 0., 0., 0., 0.)
        if self._extrap == 2:
            raise ValueError("Constant padding in 2-d needs explicit values.")
        if self._extrap == 3:
            return extrap2d_lin(arr, self._n_ext)
        if self._extrap == 4:
            return extrap2d_loglin(arr, self._n_ext)
        if self._extrap == 5:
            return extrap2d_loglin_oscil(arr, self._n_ext)
        return np.asarray(arr)

    def _axis(self, t, rows):
        """One axis: rows of pre-transform samples through transform `t`
        (its own 1-d 'outer' extension applied row by row)."""
        if t._extrap_layer == 'outer' and t._extrap:
            rows = np.array([t._perform_extrap(r) for r in rows])
        return t._transform_rows(rows)

    def transform(self, pre_samples):
        """Post-transform sample points ('ij' meshgrid) and samples."""
        pre = np.asarray(pre_samples)
        if self._extrap2d:
            pre = self._perform_extrap(pre)
        inter = self._axis(self._fbsjt[1], pre)
        post = self._axis(self._fbsjt[0], np.asarray(inter).T).T
        post = post[self._post_slice, self._post_slice]
        post_sampts = np.meshgrid(self._post_sampts, self._post_sampts,
                                  indexing='ij')
        return post_sampts, post

    def transform_cosmo_multipoles(self, direction, pre_samples):
        """Configuration <-> Fourier space double multipoles."""
        parity, prefactor = _cosmo_factors(direction, sum(self.degrees))
        post_sampts, post_samples = self.transform(pre_samples)
        return post_sampts, post_samples * (prefactor * parity)


def _resample(sampts, samples, size, spline, grid):
    sampts = np.squeeze(sampts)
    samples = np.squeeze(samples)
    if samples.ndim == 1:
        if sampts.ndim != 1:
            raise ValueError("Sample points must be 1-d.")
        res = grid(sampts[0], sampts[-1], size or len(sampts))
        return res, InterpolatedUnivariateSpline(
            sampts, samples, k=spline, ext='raise')(res)
    if samples.ndim == 2:
        if sampts.ndim == 1:
            sampts = np.array([sampts, sampts])
        if len(sampts) != 2 or np.ndim(sampts[0]) != 1 \
                or np.ndim(sampts[-1]) != 1:
            raise ValueError("Must provide (two) 1-d array(s) as sample "
                             "points for 2-d resampling.")
        size = size if isinstance(size, Sequence) else (size, size)
        res = (grid(sampts[0][0], sampts[0][-1], size[0] or len(sampts[0])),
               grid(sampts[-1][0], sampts[-1][-1],
                    size[-1] or len(sampts[-1])))
        return res, RectBivariateSpline(sampts[0], sampts[-1], samples,
                                        kx=spline, ky=spline)(*res)
    raise ValueError(f"Sample points must be 1-d or 2-d: {samples.ndim=}.")


def resample_lglin(sampts, samples, size=None, spline=3):
    """Resample at logarithmically spaced points in 1-d or 2-d (a spline of
    degree `spline` through the samples)."""
    return _resample(sampts, samples, size, spline,
                     lambda a, b, n: np.logspace(np.log10(a), np.log10(b), n))


def resample_lin(sampts, samples, size=None, spline=3):
    """Resample at linearly spaced points in 1-d or 2-d."""
    return _resample(sampts, samples, size, spline,
                     lambda a, b, n: np.linspace(a, b, n))
