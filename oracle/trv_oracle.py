"""CPU oracle: a numpy restatement of Triumvirate's mesh-based estimators.

TEST INFRASTRUCTURE ONLY.  This module is the checker for the CUDA product
path in ``triumvirate_gb300``.  Only ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py`` may import it; the product never
routes through it.

Why a restatement: the reference C++ core (``src/triumvirate/src/*.cpp``)
links GSL and FFTW3, neither of which is installed, and its Python layer
needs astropy/pyyaml, so it cannot be built or imported here.  Every
function below follows one reference function, cited as ``file:line``
relative to ``src/triumvirate/`` of MikeSWang/Triumvirate.  The third-party
arithmetic the reference takes from GSL (>=2.7) and FFTW3 (>=3.3) is
restated as:

* ``gsl_sf_coupling_3j`` -> Racah's closed formula in exact integers;
* ``gsl_sf_legendre_sphPlm`` -> ``scipy.special.lpmv`` with the
  spherical-harmonic normalisation;
* ``gsl_sf_bessel_jl`` -> ``scipy.special.spherical_jn``;
* ``gsl_spline`` (``gsl_interp_cspline``) -> natural cubic spline
  (``scipy.interpolate.CubicSpline(bc_type='natural')``, the same unique
  interpolant);
* ``fftw_plan_dft_3d`` FORWARD/BACKWARD (unnormalised, sign -1/+1) ->
  ``scipy.fft.fftn`` / ``ifftn(norm='forward')``.

Parity is pinned by the reference's own golden measurement files
(``tests/test_input/stats/*.txt``), reproduced by ``tests/test_oracle.py``
within the reference tests' tolerances.
"""
from __future__ import annotations

import math
import os
from fractions import Fraction

import numpy as np
import scipy.fft as sfft
from scipy.interpolate import CubicSpline
from scipy.special import lpmv, spherical_jn

_WORKERS = int(os.environ.get("TRVG_ORACLE_THREADS", os.cpu_count() or 1))

EPS_COUPLING = 1.e-9   # maths.cpp:165
EPS_YLM = 1.e-9        # maths.cpp:176


# ---------------------------------------------------------------------------
# Maths (maths.cpp)
# ---------------------------------------------------------------------------

def wigner_3j(j1, j2, j3, m1, m2, m3):
    """Wigner 3-j symbol (maths.cpp:167-169 -> gsl_sf_coupling_3j).

    Racah's formula evaluated in exact rational arithmetic.
    """
    if m1 + m2 + m3 != 0:
        return 0.
    if j3 < abs(j1 - j2) or j3 > j1 + j2:
        return 0.
    if abs(m1) > j1 or abs(m2) > j2 or abs(m3) > j3:
        return 0.
    f = math.factorial
    tri = Fraction(f(j1 + j2 - j3) * f(j1 - j2 + j3) * f(-j1 + j2 + j3),
                   f(j1 + j2 + j3 + 1))
    pref = tri * f(j1 + m1) * f(j1 - m1) * f(j2 + m2) * f(j2 - m2) \
        * f(j3 + m3) * f(j3 - m3)
    kmin = max(0, j2 - j3 - m1, j1 - j3 + m2)
    kmax = min(j1 + j2 - j3, j1 - m1, j2 + m2)
    s = Fraction(0)
    for k in range(kmin, kmax + 1):
        s += Fraction((-1) ** k,
                      f(k) * f(j1 + j2 - j3 - k) * f(j1 - m1 - k)
                      * f(j2 + m2 - k) * f(j3 - j2 + m1 + k)
                      * f(j3 - j1 - m2 + k))
    sign = -1 if (j1 - j2 - m3) % 2 else 1
    return sign * math.sqrt(float(pref)) * float(s)


def calc_coupling_coeff_3pt(ell1, ell2, ELL, m1, m2, M):
    """threept.cpp:65-71."""
    return float((2*ell1 + 1) * (2*ell2 + 1) * (2*ELL + 1)) \
        * wigner_3j(ell1, ell2, ELL, 0, 0, 0) \
        * wigner_3j(ell1, ell2, ELL, m1, m2, M)


def calc_coupling_coeff_2pt(ell, ELL, m, M):
    """twopt.cpp:45-49."""
    return (2*ell + 1) * (2*ELL + 1) \
        * wigner_3j(ell, 0, ELL, 0, 0, 0) * wigner_3j(ell, 0, ELL, m, 0, M)


def _sph_plm(ell, m, mu):
    """gsl_sf_legendre_sphPlm: sqrt((2l+1)/4pi (l-m)!/(l+m)!) P_l^m(mu)."""
    norm = math.sqrt((2*ell + 1) / (4*math.pi)
                     * math.factorial(ell - m) / math.factorial(ell + m))
    return norm * lpmv(m, ell, mu)


def reduced_ylm(ell, m, vec):
    """Reduced spherical harmonic on an array of 3-vectors.

    Follows ``SphericalHarmonicCalculator::calc_reduced_spherical_harmonic``
    (maths.cpp:171-220): unity for (0, 0); zero below |v| < 1e-9;
    phi = arccos(x/r_xy) reflected for y < 0; parity (-1)^m for m < 0,
    complex conjugation and the sqrt(4pi/(2l+1)) normalisation.
    """
    vec = np.asarray(vec, dtype=np.float64)
    shape = vec.shape[:-1]
    if ell == 0 and m == 0:
        return np.ones(shape, dtype=np.complex128)
    x, y, z = vec[..., 0], vec[..., 1], vec[..., 2]
    r = np.sqrt(x*x + y*y + z*z)
    safe_r = np.where(np.abs(r) < EPS_YLM, 1., r)
    mu = z / safe_r
    rxy = np.sqrt(x*x + y*y)
    safe_rxy = np.where(np.abs(rxy) >= EPS_YLM, rxy, 1.)
    phi = np.where(np.abs(rxy) >= EPS_YLM,
                   np.arccos(np.clip(x / safe_rxy, -1., 1.)), 0.)
    phi = np.where((np.abs(rxy) >= EPS_YLM) & (y < 0.), -phi + 2.*np.pi, phi)
    ylm = np.exp(1j * float(m) * phi) * _sph_plm(ell, abs(m), mu)
    ylm = float((-1) ** ((m - abs(m)) // 2)) * np.conj(ylm)
    ylm = ylm * math.sqrt(4.*math.pi / (2.*ell + 1.))
    return np.where(np.abs(r) < EPS_YLM, 0., ylm).astype(np.complex128)


class SphericalBessel:
    """``SphericalBesselCalculator`` (maths.cpp:309-375, maths.hpp:305-306).

    Natural cubic spline of j_ell on x = 0.05 i over [0, max(1000, ell^2)];
    direct evaluation at and beyond the split point.
    """

    def __init__(self, ell):
        self.ell = ell
        self.split = 1000. if 1000. >= ell * ell else float(ell * ell)
        step = 0.05
        nsample = int((self.split - 0.) / step) + 1
        xs = 0. + step * np.arange(nsample, dtype=np.float64)
        self._spline = CubicSpline(xs, spherical_jn(ell, xs),
                                   bc_type='natural')

    def eval(self, x):
        x = np.asarray(x, dtype=np.float64)
        out = np.empty_like(x)
        hi = x >= self.split
        out[~hi] = self._spline(x[~hi])
        if hi.any():
            out[hi] = spherical_jn(self.ell, x[hi])
        return out


# ---------------------------------------------------------------------------
# Parameters and binning (parameters.cpp, dataobjs.cpp)
# ---------------------------------------------------------------------------

_ORDER = {'ngp': 1, 'cic': 2, 'tsc': 3, 'pcs': 4}


class Params:
    """Derived parameters (parameters.cpp:466-1270, subset on the path)."""

    def __init__(self, boxsize, ngrid, assignment='tsc', interlace=False,
                 ell1=0, ell2=0, ELL=0, form='diag', idx_bin=0,
                 npoint='3pt'):
        self.boxsize = np.array(
            [boxsize] * 3 if np.isscalar(boxsize) else boxsize, dtype=float)
        self.ngrid = np.array(
            [ngrid] * 3 if np.isscalar(ngrid) else ngrid, dtype=np.int64)
        self.assignment = assignment
        self.assignment_order = _ORDER[assignment]     # parameters.cpp:660-669
        # parameters.cpp:1240-1249: no interlacing for 3-pt statistics.
        self.interlace = bool(interlace) and npoint != '3pt'
        self.ell1, self.ell2, self.ELL = int(ell1), int(ell2), int(ELL)
        self.form = form
        # parameters.cpp:829-848: 'full' with ell1 == ell2 -> 'triu'.
        self.shape = 'triu' if (form == 'full' and ell1 == ell2) else form
        self.idx_bin = 0 if idx_bin is None else int(idx_bin)
        self.volume = float(self.boxsize[0] * self.boxsize[1]
                            * self.boxsize[2])        # parameters.cpp:1028
        self.nmesh = int(self.ngrid[0] * self.ngrid[1] * self.ngrid[2])
        self.vol_cell = self.volume / float(self.nmesh)   # field.cpp:364


def lin_binning(bin_min, bin_max, num_bins):
    """``Binning::compute_binning`` 'lin' scheme (dataobjs.cpp:148-158)."""
    dbin = (bin_max - bin_min) / float(num_bins)
    edges, centres = [], []
    for i in range(num_bins):
        left = bin_min + dbin * i
        edges.append(left)
        centres.append(left + dbin / 2.)
    edges.append(bin_max)
    return np.array(edges), np.array(centres)


# ---------------------------------------------------------------------------
# Mesh field (field.cpp)
# ---------------------------------------------------------------------------

def _axis_stencil(loc, n, order, shadow):
    """Per-axis cell indices and weights of one assignment scheme.

    NGP field.cpp:639-653, CIC 749-764, TSC 860-891 (shadow 926-960),
    PCS 1008-1032.
    """
    idx = np.trunc(loc).astype(np.int64)
    s = loc - idx
    npart = loc.shape[0]
    ijk = np.zeros((order, npart), dtype=np.int64)
    win = np.zeros((order, npart), dtype=np.float64)
    if order == 1:
        up = (loc - idx) >= 0.5
        ijk[0] = np.where(up, np.where(idx == n - 1, 0, idx + 1), idx)
        win[0] = 1.
    elif order == 2:
        ijk[0] = idx
        ijk[1] = np.where(idx == n - 1, 0, idx + 1)
        win[0] = 1. - s
        win[1] = s
    elif order == 3:
        lo = s < 0.5
        a0 = np.where(idx == 0, n - 1, idx - 1)
        a2 = np.where(idx == n - 1, 0, idx + 1)
        b1 = np.where(idx == n - 1, 0, idx + 1)
        if shadow:
            # field.cpp:940-945 (as written in the reference's shadow pass).
            b2 = np.where(idx == n - 1, 0, b1 + 1)
        else:
            b2 = np.where(b1 == n - 1, 0, b1 + 1)
        ijk[0] = np.where(lo, a0, idx)
        ijk[1] = np.where(lo, idx, b1)
        ijk[2] = np.where(lo, a2, b2)
        sl = s
        sh = 1. - s
        win[0] = np.where(lo, 0.5 * (0.5 - sl) * (0.5 - sl),
                          0.5 * (0.5 + sh) * (0.5 + sh))
        win[1] = np.where(lo, 0.75 - sl * sl, 0.75 - sh * sh)
        win[2] = np.where(lo, 0.5 * (0.5 + sl) * (0.5 + sl),
                          0.5 * (0.5 - sh) * (0.5 - sh))
    elif order == 4:
        ijk[0] = np.where(idx == 0, n - 1, idx - 1)
        ijk[1] = idx
        ijk[2] = np.where(idx == n - 1, 0, idx + 1)
        ijk[3] = np.where(ijk[2] == n - 1, 0, ijk[2] + 1)
        t = 1. - s
        win[0] = 1./6 * t * t * t
        win[1] = 1./6 * (4. - 6. * s * s + 3. * s * s * s)
        win[2] = 1./6 * (4. - 6. * t * t + 3. * t * t * t)
        win[3] = 1./6 * s * s * s
    return ijk, win


def assign_weighted_field_to_mesh(pos, weight, params, shadow=False):
    """``MeshField::assign_weighted_field_to_mesh_*`` (field.cpp:569-1112).

    Returns the complex128 mesh sum_i w_i W(x - x_i) / dV.  With
    ``shadow`` the half-cell-shifted interlacing mesh is returned.
    """
    pos = np.asarray(pos, dtype=np.float64)
    weight = np.asarray(weight, dtype=np.complex128)
    order = params.assignment_order
    ng = params.ngrid
    inv_vol_cell = 1. / params.vol_cell
    ijks, wins = [], []
    for ax in range(3):
        loc = ng[ax] * pos[:, ax] / params.boxsize[ax]
        if shadow:
            loc = loc + 0.5
            loc = np.where(loc > ng[ax], loc - ng[ax], loc)
        ijk, win = _axis_stencil(loc, int(ng[ax]), order, shadow)
        ijks.append(ijk)
        wins.append(win)
    mesh = np.zeros(params.nmesh, dtype=np.complex128)
    for a in range(order):
        for b in range(order):
            for c in range(order):
                gid = (ijks[0][a] * ng[1] + ijks[1][b]) * ng[2] + ijks[2][c]
                val = inv_vol_cell * weight.real * wins[0][a] \
                    * wins[1][b] * wins[2][c] \
                    + 1j * (inv_vol_cell * weight.imag * wins[0][a]
                            * wins[1][b] * wins[2][c])
                ok = (gid >= 0) & (gid < params.nmesh)
                np.add.at(mesh, gid[ok], val[ok])
    return mesh.reshape(tuple(ng))


class Mesh:
    """A mesh field with its optional interlacing shadow."""

    def __init__(self, field, shadow=None):
        self.field = field
        self.shadow = shadow


def mesh_weighted(pos, weight, params):
    """Assignment of one catalogue with the shadow pass when interlacing."""
    f = assign_weighted_field_to_mesh(pos, weight, params)
    s = assign_weighted_field_to_mesh(pos, weight, params, shadow=True) \
        if params.interlace else None
    return Mesh(f, s)


def _fftn(a):
    return sfft.fftn(a, workers=_WORKERS)


def _ifftn_unnorm(a):
    return sfft.ifftn(a, norm='forward', workers=_WORKERS)


def _shifted_indices(n):
    i = np.arange(n)
    return np.where(i < n // 2, i, i - n)


def grid_wavevectors(params):
    """``MeshField::get_grid_wavevector`` (field.cpp:555-562) on all cells."""
    dk = 2. * np.pi / params.boxsize
    kx = _shifted_indices(params.ngrid[0]) * dk[0]
    ky = _shifted_indices(params.ngrid[1]) * dk[1]
    kz = _shifted_indices(params.ngrid[2]) * dk[2]
    KX, KY, KZ = np.meshgrid(kx, ky, kz, indexing='ij')
    return KX, KY, KZ


def grid_positions(params):
    """``MeshField::get_grid_pos_vector`` (field.cpp:545-552)."""
    dr = params.boxsize / params.ngrid
    rx = _shifted_indices(params.ngrid[0]) * dr[0]
    ry = _shifted_indices(params.ngrid[1]) * dr[1]
    rz = _shifted_indices(params.ngrid[2]) * dr[2]
    return np.meshgrid(rx, ry, rz, indexing='ij')


def vec3_mag(x, y, z):
    """maths.cpp:57-59 (left-to-right sum, then sqrt)."""
    return np.sqrt(x * x + y * y + z * z)


def fourier_transform(mesh, params):
    """``MeshField::fourier_transform`` (field.cpp:1496-1655)."""
    f = _fftn(mesh.field * params.vol_cell)
    if params.interlace:
        fs = _fftn(mesh.shadow * params.vol_cell)
        ng = params.ngrid
        m = [np.where(np.arange(n) < n // 2, np.arange(n) / float(n),
                      np.arange(n) / float(n) - 1) for n in ng]
        MX, MY, MZ = np.meshgrid(*m, indexing='ij')
        arg = np.pi * (MX + MY + MZ)
        f = (f + (np.cos(arg) + 1j * np.sin(arg)) * fs) / 2.
    return f


def assignment_window(params, order=None):
    """``MeshField::calc_assignment_window_in_fourier`` (field.cpp:1114-1146)."""
    order = params.assignment_order if order is None else order
    ws = []
    for n in params.ngrid:
        i = _shifted_indices(n)
        u = np.pi * i / float(n)
        with np.errstate(invalid='ignore', divide='ignore'):
            w = np.where(i != 0, np.sin(u) / np.where(i != 0, u, 1.), 1.)
        ws.append(w)
    WX, WY, WZ = np.meshgrid(*ws, indexing='ij')
    return (WX * WY * WZ) ** order


def shotnoise_aliasing(params):
    """``FieldStats::calc_shotnoise_aliasing_*`` (field.cpp:3403-3564)."""
    ng = params.ngrid
    us = [np.pi * _shifted_indices(n) / float(n) for n in ng]
    UX, UY, UZ = np.meshgrid(*us, indexing='ij')
    if params.interlace:
        uhalf = np.sqrt(UX * UX + UY * UY + UZ * UZ) / 2.
        s2h = np.sin(uhalf) * np.sin(uhalf)
        c2h = np.cos(uhalf) * np.cos(uhalf)
        p = params.assignment_order
        cc = c2h ** p
        if p == 2:
            cs = 1. - 2./3. * s2h
        elif p == 3:
            cs = 1. - s2h + 2./15. * s2h * s2h
        elif p == 4:
            cs = 1. - 4./3. * s2h + 2./5. * s2h * s2h \
                - 4./315. * s2h * s2h * s2h
        else:
            cs = np.ones_like(s2h)
        return cc * cs
    IX, IY, IZ = np.meshgrid(*[_shifted_indices(n) for n in ng],
                             indexing='ij')
    s2 = [np.where(I != 0, np.sin(U) * np.sin(U), 0.)
          for I, U in ((IX, UX), (IY, UY), (IZ, UZ))]
    a = params.assignment
    if a == 'ngp':
        return np.ones(tuple(ng))
    if a == 'cic':
        f = [1. - 2./3. * s for s in s2]
    elif a == 'tsc':
        f = [1. - s + 2./15. * s * s for s in s2]
    else:
        f = [1. - 4./3. * s + 2./5. * s * s - 4./315. * s * s * s for s in s2]
    return f[0] * f[1] * f[2]


def inv_fourier_transform(fk, params):
    """``MeshField::inv_fourier_transform`` (field.cpp:1657-1720)."""
    return _ifftn_unnorm(fk / params.volume)


def band_limited_ifft(fk, ylm_k, win, kmag, k_lower, k_upper):
    """``inv_fourier_transform_ylm_wgtd_field_band_limited``
    (field.cpp:1792-1906).  Returns (F(x), k_eff, nmodes)."""
    sel = (k_lower <= kmag) & (kmag < k_upper)
    nmodes = int(np.count_nonzero(sel))
    k_eff = float(np.sum(kmag[sel]))
    g = np.where(sel, ylm_k * (fk / win), 0.)
    F = _ifftn_unnorm(g)
    F = F / float(nmodes)
    return F, k_eff / float(nmodes), nmodes


def sjl_ylm_ifft(fk, ylm_k, win, kmag, sjl, r, params):
    """``inv_fourier_transform_sjl_ylm_wgtd_field`` (field.cpp:1908-2010)."""
    j = sjl.eval((kmag * r).ravel()).reshape(kmag.shape)
    g = j * (ylm_k * (fk / win)) / params.volume
    return _ifftn_unnorm(g)


def twopt_stats_in_fourier(fa, fb, shotnoise_amp, ell, m, edges, centres,
                           params, kvec, kmag, win_pk, alias):
    """``FieldStats::compute_ylm_wgtd_2pt_stats_in_fourier``
    (field.cpp:2511-2703): fine binning at dk = 1e-5 (1e6 samples), then
    bins collect the samples whose left edge i*dk lies in them."""
    n_sample = 1000000
    dk_sample = 1.e-5
    idx_k = np.trunc(kmag / dk_sample).astype(np.int64)
    ok = (idx_k >= 0) & (idx_k < n_sample)
    ylm = reduced_ylm(ell, m, np.stack(kvec, axis=-1))
    pk_mode = fa * np.conj(fb) / win_pk * ylm
    sn_mode = shotnoise_amp * alias / (win_pk if params.interlace else alias)
    sn_mode = sn_mode * ylm
    idx = idx_k[ok]
    nm = np.bincount(idx, minlength=n_sample)
    ks = np.bincount(idx, weights=kmag[ok], minlength=n_sample)
    pr = np.bincount(idx, weights=pk_mode.real[ok], minlength=n_sample)
    pi = np.bincount(idx, weights=pk_mode.imag[ok], minlength=n_sample)
    sr = np.bincount(idx, weights=sn_mode.real[ok], minlength=n_sample)
    si = np.bincount(idx, weights=sn_mode.imag[ok], minlength=n_sample)
    ksample = np.arange(n_sample) * dk_sample
    nb = len(centres)
    out = dict(nmodes=np.zeros(nb, np.int64), k=np.zeros(nb),
               pk=np.zeros(nb, np.complex128), sn=np.zeros(nb, np.complex128))
    for b in range(nb):
        sel = (edges[b] <= ksample) & (ksample < edges[b + 1])
        n = int(nm[sel].sum())
        out['nmodes'][b] = n
        if n != 0:
            out['k'][b] = ks[sel].sum() / n
            out['pk'][b] = (pr[sel].sum() + 1j * pi[sel].sum()) / n
            out['sn'][b] = (sr[sel].sum() + 1j * si[sel].sum()) / n
        else:
            out['k'][b] = centres[b]
    return out


def twopt_field(fa, fb, shotnoise_amp, params, win_pk, alias):
    """Common first half of the uncoupled shot-noise routines
    (field.cpp:3288-3345 / 3010-3070): IFFT of (fa fb^* / W - S C1 / W) / V."""
    win_sn = win_pk if params.interlace else alias
    pk = fa * np.conj(fb) / win_pk - shotnoise_amp * alias / win_sn
    return _ifftn_unnorm(pk / params.volume)


def shotnoise_bispec_per_bin(xi, ylm_a, ylm_b, sj_a, sj_b, rmag, k_a, k_b,
                             params):
    """``compute_uncoupled_shotnoise_for_bispec_per_bin``
    (field.cpp:3349-3396): vol_cell * sum_x j_a j_b y_a y_b xi(x)."""
    ja = sj_a.eval((k_a * rmag).ravel()).reshape(rmag.shape)
    jb = sj_b.eval((k_b * rmag).ravel()).reshape(rmag.shape)
    return complex(np.sum(xi * (ja * jb * ylm_a * ylm_b))) * params.vol_cell


def shotnoise_3pcf(xi, ylm_a, ylm_b, rmag, edges, centres, params):
    """``compute_uncoupled_shotnoise_for_3pcf`` (field.cpp:3090-3196)."""
    n_sample = 100000
    dr_sample = 1.
    idx_r = np.trunc(rmag / dr_sample).astype(np.int64)
    ok = (idx_r >= 0) & (idx_r < n_sample)
    val = xi * ylm_a * ylm_b
    idx = idx_r[ok]
    npairs_s = np.bincount(idx, minlength=n_sample)
    r_s = np.bincount(idx, weights=rmag[ok], minlength=n_sample)
    xr = np.bincount(idx, weights=val.real[ok], minlength=n_sample)
    xim = np.bincount(idx, weights=val.imag[ok], minlength=n_sample)
    rsample = np.arange(n_sample) * dr_sample
    nb = len(centres)
    npairs = np.zeros(nb, np.int64)
    r = np.zeros(nb)
    xi_b = np.zeros(nb, np.complex128)
    for b in range(nb):
        sel = (edges[b] <= rsample) & (rsample < edges[b + 1])
        n = int(npairs_s[sel].sum())
        npairs[b] = n
        if n != 0:
            r[b] = r_s[sel].sum() / n
            xi_b[b] = (xr[sel].sum() + 1j * xim[sel].sum()) / n
        else:
            r[b] = centres[b]
    norm = 1. / params.vol_cell * (-1.) ** (params.ell1 + params.ell2)
    for b in range(nb):
        if npairs[b] != 0:
            xi_b[b] *= norm / float(npairs[b])
    return npairs, r, xi_b


def ylm_grid(ell, m, vecs):
    return reduced_ylm(ell, m, np.stack(vecs, axis=-1))


# ---------------------------------------------------------------------------
# Data-vector layout helpers (threept.cpp: per-shape index arithmetic)
# ---------------------------------------------------------------------------

def dv_pairs(shape, num_bins, idx_bin):
    """Bin pairs (row, col) in data-vector order for each form
    (threept.cpp:1675-1968)."""
    if shape == 'diag':
        return [(b, b) for b in range(num_bins)]
    if shape == 'off-diag':
        d = abs(idx_bin)
        if idx_bin >= 0:
            return [(i, i + d) for i in range(num_bins - d)]
        return [(i + d, i) for i in range(num_bins - d)]
    if shape == 'row':
        return [(idx_bin, c) for c in range(num_bins)]
    if shape == 'full':
        return [(r, c) for r in range(num_bins) for c in range(num_bins)]
    if shape == 'triu':
        return [(r, c) for r in range(num_bins) for c in range(r, num_bins)]
    raise ValueError(f"unrecognised shape {shape}")


def _sn_single_leg(shape, pairs, S_bins, factor_mirror, leg):
    """Shot-noise single-leg contributions S_i_jk / S_ik_j per data-vector
    entry (threept.cpp:1981-2126).  The 'full' ell1 = 0 branch in the
    reference loops one row past the data vector (threept.cpp:2103); only
    in-range entries are accumulated here."""
    out = np.zeros(len(pairs), np.complex128)
    for i, (r, c) in enumerate(pairs):
        b = r if leg == 0 else c
        S = S_bins[b]
        out[i] = S + factor_mirror * np.conj(S)
    return out


# ---------------------------------------------------------------------------
# Estimators (threept.cpp, twopt.cpp)
# ---------------------------------------------------------------------------

def _sph_orders_gpp(params):
    """Non-redundant (m1, m2, 0) with nonzero coupling
    (threept.cpp:1580-1601)."""
    done, out = [], []
    for m1 in range(-params.ell1, params.ell1 + 1):
        for m2 in range(-params.ell2, params.ell2 + 1):
            M = 0
            if any(m1 + a == 0 and m2 + b == 0 and M + c == 0
                   for (a, b, c) in done):
                continue
            coupling = calc_coupling_coeff_3pt(params.ell1, params.ell2,
                                               params.ELL, m1, m2, M)
            if abs(coupling) < EPS_COUPLING:
                continue
            out.append((m1, m2, M, coupling))
            done.append((m1, m2, M))
    return out


def _sph_orders_lpp(params):
    """Non-redundant (m1, m2, M) for the local plane-parallel estimator
    (threept.cpp:354-404)."""
    done, out = [], []
    for m1 in range(-params.ell1, params.ell1 + 1):
        for m2 in range(-params.ell2, params.ell2 + 1):
            if all(abs(calc_coupling_coeff_3pt(params.ell1, params.ell2,
                                               params.ELL, m1, m2, M))
                   <= EPS_COUPLING
                   for M in range(-params.ELL, params.ELL + 1)):
                continue
            for M in range(-params.ELL, params.ELL + 1):
                if any(m1 + a == 0 and m2 + b == 0 and M + c == 0
                       for (a, b, c) in done):
                    continue
                coupling = calc_coupling_coeff_3pt(params.ell1, params.ell2,
                                                   params.ELL, m1, m2, M)
                if abs(coupling) < EPS_COUPLING:
                    continue
                out.append((m1, m2, M, coupling))
                done.append((m1, m2, M))
    return out


def _validate_coupling(params):
    """threept.cpp:73-89."""
    if abs(wigner_3j(params.ell1, params.ell2, params.ELL, 0, 0, 0)) \
            < EPS_COUPLING:
        raise ValueError("Specified three-point correlator multipole "
                         "vanishes identically owing to zero-valued "
                         "Wigner 3-j symbol.")


def _unit_mesh_fluct(pos, params):
    """``compute_unweighted_field_fluctuations_insitu``
    (field.cpp:1229-1244): unit weights, then subtract N/V (main mesh)."""
    w = np.ones(pos.shape[0], dtype=np.complex128)
    m = mesh_weighted(pos, w, params)
    m.field = m.field - float(pos.shape[0]) / params.volume
    return m


def _unit_mesh(pos, params):
    """``compute_unweighted_field`` (field.cpp:1208-1227)."""
    w = np.ones(pos.shape[0], dtype=np.complex128)
    return mesh_weighted(pos, w, params)


def compute_bispec_in_gpp_box(pos, params, edges, centres, norm_factor):
    """``trv::compute_bispec_in_gpp_box`` (threept.cpp:1473-2188)."""
    _validate_coupling(params)
    pairs = dv_pairs(params.shape, len(centres), params.idx_bin)
    ndv = len(pairs)
    factor_phase = (1j) ** (params.ell1 + params.ell2)
    npart = pos.shape[0]

    dn_k = fourier_transform(_unit_mesh_fluct(pos, params), params)
    N_k = fourier_transform(_unit_mesh(pos, params), params)
    win = assignment_window(params)
    alias = shotnoise_aliasing(params)
    win_pk = (win * win) if params.interlace else alias
    kvec = grid_wavevectors(params)
    kmag = vec3_mag(*kvec)
    rvec = grid_positions(params)
    rmag = vec3_mag(*rvec)
    sj_a = SphericalBessel(params.ell1)
    sj_b = SphericalBessel(params.ell2)

    out = _empty_dv(ndv)
    for term_idx, (m1, m2, M, coupling) in enumerate(_sph_orders_gpp(params)):
        zero = (m1 == 0 and m2 == 0 and M == 0)
        factor_mirror = 0. if zero else (-1.) ** params.ELL
        factor_mirror_w3j = 0. if zero else 1.
        ylm_k_a = ylm_grid(params.ell1, m1, kvec)
        ylm_k_b = ylm_grid(params.ell2, m2, kvec)
        ylm_r_a = ylm_grid(params.ell1, m1, rvec)
        ylm_r_b = ylm_grid(params.ell2, m2, rvec)

        # G_00 (threept.cpp:1665-1670).
        G = inv_fourier_transform(dn_k / win, params)

        _raw_pairs(out, pairs, edges, centres, dn_k, ylm_k_a, ylm_k_b, win,
                   kmag, G, coupling, params.vol_cell, factor_mirror,
                   term_idx == 0)

        # Shot noise (threept.cpp:1974-2140).
        Sbar = complex(float(npart))
        if params.ell1 == 0 and params.ell2 == 0:
            out['sn'] += coupling * Sbar
        if params.ell2 == 0:
            st = twopt_stats_in_fourier(dn_k, N_k, Sbar, params.ell1, m1,
                                        edges, centres, params, kvec, kmag,
                                        win_pk, alias)
            S = coupling * (st['pk'] - st['sn'])
            out['sn'] += _sn_single_leg(params.shape, pairs, S,
                                        factor_mirror, 0)
        if params.ell1 == 0:
            st = twopt_stats_in_fourier(dn_k, N_k, Sbar, params.ell2, m2,
                                        edges, centres, params, kvec, kmag,
                                        win_pk, alias)
            S = coupling * (st['pk'] - st['sn'])
            out['sn'] += _sn_single_leg(params.shape, pairs, S,
                                        factor_mirror, 1)
        xi = twopt_field(dn_k, N_k, Sbar, params, win_pk, alias)
        for i in range(ndv):
            S_ij_k = coupling * shotnoise_bispec_per_bin(
                xi, ylm_r_a, ylm_r_b, sj_a, sj_b, rmag,
                out['k1_eff'][i], out['k2_eff'][i], params)
            out['sn'][i] += factor_phase * (
                S_ij_k + factor_mirror_w3j * np.conj(S_ij_k))
    return _finish_bispec(out, norm_factor)


def _empty_dv(ndv):
    return dict(k1_bin=np.zeros(ndv), k2_bin=np.zeros(ndv),
                k1_eff=np.zeros(ndv), k2_eff=np.zeros(ndv),
                nmodes_1=np.zeros(ndv, np.int64),
                nmodes_2=np.zeros(ndv, np.int64),
                bk=np.zeros(ndv, np.complex128),
                sn=np.zeros(ndv, np.complex128))


def _raw_pairs(out, pairs, edges, centres, dn_k, ylm_k_a, ylm_k_b, win,
               kmag, G, coupling, vol_cell, factor_mirror, first_term):
    """Per-pair band-limited IFFTs and triple-product reduction
    (threept.cpp:1675-1968)."""
    for i, (ra, cb) in enumerate(pairs):
        Fa, keff_a, nm_a = band_limited_ifft(dn_k, ylm_k_a, win, kmag,
                                             edges[ra], edges[ra + 1])
        Fb, keff_b, nm_b = band_limited_ifft(dn_k, ylm_k_b, win, kmag,
                                             edges[cb], edges[cb + 1])
        if first_term:
            out['k1_bin'][i] = centres[ra]
            out['k2_bin'][i] = centres[cb]
            out['k1_eff'][i] = keff_a
            out['k2_eff'][i] = keff_b
            out['nmodes_1'][i] = nm_a
            out['nmodes_2'][i] = nm_b
        comp = complex(np.sum(Fa * Fb * G))
        out['bk'][i] += coupling * vol_cell * (
            comp + factor_mirror * np.conj(comp))


def _finish_bispec(out, norm_factor):
    return dict(k1_bin=out['k1_bin'], k1_eff=out['k1_eff'],
                nmodes_1=out['nmodes_1'], k2_bin=out['k2_bin'],
                k2_eff=out['k2_eff'], nmodes_2=out['nmodes_2'],
                bk_raw=norm_factor * out['bk'],
                bk_shot=norm_factor * out['sn'])


def _ylm_weights(ell, m, los, w, power=1, conj=False):
    y = reduced_ylm(ell, m, los)
    if conj:
        y = np.conj(y)
    return y * w ** power


def _ylm_wgtd_field(pos_d, los_d, w_d, pos_r, los_r, w_r, alpha, ell, m,
                    params):
    """``compute_ylm_wgtd_field`` data - alpha rand (field.cpp:1246-1323)."""
    md = mesh_weighted(pos_d, _ylm_weights(ell, m, los_d, w_d), params)
    mr = mesh_weighted(pos_r, _ylm_weights(ell, m, los_r, w_r), params)
    f = md.field - alpha * mr.field
    s = (md.shadow - alpha * mr.shadow) if params.interlace else None
    return Mesh(f, s)


def _ylm_wgtd_quad_field(pos_d, los_d, w_d, pos_r, los_r, w_r, alpha, ell,
                         m, params):
    """``compute_ylm_wgtd_quad_field`` data + alpha^2 rand
    (field.cpp:1364-1443)."""
    md = mesh_weighted(pos_d, _ylm_weights(ell, m, los_d, w_d, 2, True),
                       params)
    mr = mesh_weighted(pos_r, _ylm_weights(ell, m, los_r, w_r, 2, True),
                       params)
    f = md.field + alpha ** 2 * mr.field
    s = (md.shadow + alpha ** 2 * mr.shadow) if params.interlace else None
    return Mesh(f, s)


def shotnoise_amp_bispec(los_d, w_d, los_r, w_r, alpha, ell, m):
    """``calc_ylm_wgtd_shotnoise_amp_for_bispec`` (threept.cpp:156-208)."""
    sd = np.sum(reduced_ylm(ell, m, los_d) * w_d ** 3)
    sr = np.sum(reduced_ylm(ell, m, los_r) * w_r ** 3)
    return complex(sd + alpha ** 3 * sr)


def shotnoise_amp_powspec(los_d, w_d, los_r, w_r, alpha, ell, m):
    """``calc_ylm_wgtd_shotnoise_amp_for_powspec`` (twopt.cpp:298-350)."""
    sd = np.sum(reduced_ylm(ell, m, los_d) * w_d ** 2)
    sr = np.sum(reduced_ylm(ell, m, los_r) * w_r ** 2)
    return complex(sd + alpha ** 2 * sr)


def compute_bispec(data, rand, params, edges, centres, norm_factor):
    """``trv::compute_bispec`` (threept.cpp:248-1012).

    ``data``/``rand`` are dicts with 'pos' (n,3), 'los' (n,3), 'w', 'ws'.
    """
    _validate_coupling(params)
    alpha = float(np.sum(data['ws'])) / float(np.sum(rand['ws']))
    pairs = dv_pairs(params.shape, len(centres), params.idx_bin)
    ndv = len(pairs)
    factor_phase = (1j) ** (params.ell1 + params.ell2)
    args = (data['pos'], data['los'], data['w'], rand['pos'], rand['los'],
            rand['w'], alpha)

    dn_00 = fourier_transform(_ylm_wgtd_field(*args, 0, 0, params), params)
    N_00 = fourier_transform(_ylm_wgtd_quad_field(*args, 0, 0, params),
                             params)
    win = assignment_window(params)
    alias = shotnoise_aliasing(params)
    win_pk = (win * win) if params.interlace else alias
    kvec = grid_wavevectors(params)
    kmag = vec3_mag(*kvec)
    rvec = grid_positions(params)
    rmag = vec3_mag(*rvec)
    sj_a = SphericalBessel(params.ell1)
    sj_b = SphericalBessel(params.ell2)

    out = _empty_dv(ndv)
    for term_idx, (m1, m2, M, coupling) in enumerate(_sph_orders_lpp(params)):
        zero = (m1 == 0 and m2 == 0 and M == 0)
        factor_mirror = 0. if zero else (-1.) ** params.ELL
        factor_mirror_w3j = 0. if zero else 1.
        ylm_k_a = ylm_grid(params.ell1, m1, kvec)
        ylm_k_b = ylm_grid(params.ell2, m2, kvec)
        ylm_r_a = ylm_grid(params.ell1, m1, rvec)
        ylm_r_b = ylm_grid(params.ell2, m2, rvec)

        G_k = fourier_transform(
            _ylm_wgtd_field(*args, params.ELL, M, params), params)
        G = inv_fourier_transform(G_k / win, params)
        _raw_pairs(out, pairs, edges, centres, dn_00, ylm_k_a, ylm_k_b, win,
                   kmag, G, coupling, params.vol_cell, factor_mirror,
                   term_idx == 0)

        dn_LM = G_k   # same field before compensation (threept.cpp:777-784)
        N_LM = fourier_transform(
            _ylm_wgtd_quad_field(*args, params.ELL, M, params), params)
        Sbar = shotnoise_amp_bispec(data['los'], data['w'], rand['los'],
                                    rand['w'], alpha, params.ELL, M)
        if params.ell1 == 0 and params.ell2 == 0:
            out['sn'] += coupling * Sbar
        if params.ell2 == 0:
            st = twopt_stats_in_fourier(dn_00, N_LM, Sbar, params.ell1, m1,
                                        edges, centres, params, kvec, kmag,
                                        win_pk, alias)
            S = coupling * (st['pk'] - st['sn'])
            out['sn'] += _sn_single_leg(params.shape, pairs, S,
                                        factor_mirror, 0)
        if params.ell1 == 0:
            st = twopt_stats_in_fourier(dn_00, N_LM, Sbar, params.ell2, m2,
                                        edges, centres, params, kvec, kmag,
                                        win_pk, alias)
            S = coupling * (st['pk'] - st['sn'])
            out['sn'] += _sn_single_leg(params.shape, pairs, S,
                                        factor_mirror, 1)
        xi = twopt_field(dn_LM, N_00, Sbar, params, win_pk, alias)
        for i in range(ndv):
            S_ij_k = coupling * shotnoise_bispec_per_bin(
                xi, ylm_r_a, ylm_r_b, sj_a, sj_b, rmag,
                out['k1_eff'][i], out['k2_eff'][i], params)
            out['sn'][i] += factor_phase * (
                S_ij_k + factor_mirror_w3j * np.conj(S_ij_k))
    return _finish_bispec(out, norm_factor)


def _empty_3pcf(ndv):
    return dict(r1_bin=np.zeros(ndv), r2_bin=np.zeros(ndv),
                r1_eff=np.zeros(ndv), r2_eff=np.zeros(ndv),
                npairs_1=np.zeros(ndv, np.int64),
                npairs_2=np.zeros(ndv, np.int64),
                zeta=np.zeros(ndv, np.complex128),
                sn=np.zeros(ndv, np.complex128))


def _sn_3pcf_diag_entries(shape, pairs, num_bins, idx_bin):
    """Data-vector entries that receive the S_ij_k term of the 3PCF
    (threept.cpp:2307-2345): only r1 = r2 entries."""
    out = []
    for i, (r, c) in enumerate(pairs):
        if shape == 'off-diag' and idx_bin != 0:
            continue
        if r == c:
            out.append((i, r))
    return out


def _zeta_pairs(out, pairs, centres, npairs, r_eff, first_term):
    if first_term:
        for i, (r, c) in enumerate(pairs):
            out['r1_bin'][i] = centres[r]
            out['r2_bin'][i] = centres[c]
            out['r1_eff'][i] = r_eff[r]
            out['r2_eff'][i] = r_eff[c]
            out['npairs_1'][i] = npairs[r]
            out['npairs_2'][i] = npairs[c]


def compute_3pcf_in_gpp_box(pos, params, edges, centres, norm_factor):
    """``trv::compute_3pcf_in_gpp_box`` (threept.cpp:2190-2619)."""
    _validate_coupling(params)
    pairs = dv_pairs(params.shape, len(centres), params.idx_bin)
    ndv = len(pairs)
    factor_phase = (1j) ** (params.ell1 + params.ell2)
    factor_parity = (-1.) ** (params.ell1 + params.ell2)
    npart = pos.shape[0]
    dn_k = fourier_transform(_unit_mesh_fluct(pos, params), params)
    N_k = fourier_transform(_unit_mesh(pos, params), params)
    win = assignment_window(params)
    alias = shotnoise_aliasing(params)
    win_pk = (win * win) if params.interlace else alias
    kvec = grid_wavevectors(params)
    kmag = vec3_mag(*kvec)
    rvec = grid_positions(params)
    rmag = vec3_mag(*rvec)
    sj_a = SphericalBessel(params.ell1)
    sj_b = SphericalBessel(params.ell2)
    out = _empty_3pcf(ndv)
    for term_idx, (m1, m2, M, coupling) in enumerate(_sph_orders_gpp(params)):
        zero = (m1 == 0 and m2 == 0 and M == 0)
        factor_mirror = 0. if zero else (-1.) ** params.ELL
        factor_mirror_w3j = 0. if zero else 1.
        ylm_r_a = ylm_grid(params.ell1, m1, rvec)
        ylm_r_b = ylm_grid(params.ell2, m2, rvec)
        ylm_k_a = ylm_grid(params.ell1, m1, kvec)
        ylm_k_b = ylm_grid(params.ell2, m2, kvec)
        xi = twopt_field(dn_k, N_k, complex(float(npart)), params, win_pk,
                         alias)
        npairs, r_eff, xi_b = shotnoise_3pcf(xi, ylm_r_a, ylm_r_b, rmag,
                                             edges, centres, params)
        for i, b in _sn_3pcf_diag_entries(params.shape, pairs, len(centres),
                                          params.idx_bin):
            out['sn'][i] += coupling * factor_parity * (
                xi_b[b] + factor_mirror_w3j * np.conj(xi_b[b]))
        _zeta_pairs(out, pairs, centres, npairs, r_eff, term_idx == 0)
        G = inv_fourier_transform(dn_k / win, params)
        for i in range(ndv):
            Fa = sjl_ylm_ifft(dn_k, ylm_k_a, win, kmag, sj_a,
                              out['r1_eff'][i], params)
            Fb = sjl_ylm_ifft(dn_k, ylm_k_b, win, kmag, sj_b,
                              out['r2_eff'][i], params)
            comp = complex(np.sum(Fa * Fb * G))
            out['zeta'][i] += coupling * params.vol_cell * factor_phase * (
                comp + factor_mirror * np.conj(comp))
    return _finish_3pcf(out, norm_factor)


def _finish_3pcf(out, norm_factor):
    return dict(r1_bin=out['r1_bin'], r1_eff=out['r1_eff'],
                npairs_1=out['npairs_1'], r2_bin=out['r2_bin'],
                r2_eff=out['r2_eff'], npairs_2=out['npairs_2'],
                zeta_raw=norm_factor * out['zeta'],
                zeta_shot=norm_factor * out['sn'])


def compute_3pcf(data, rand, params, edges, centres, norm_factor):
    """``trv::compute_3pcf`` (threept.cpp:1014-1471)."""
    _validate_coupling(params)
    alpha = float(np.sum(data['ws'])) / float(np.sum(rand['ws']))
    pairs = dv_pairs(params.shape, len(centres), params.idx_bin)
    ndv = len(pairs)
    factor_phase = (1j) ** (params.ell1 + params.ell2)
    factor_parity = (-1.) ** (params.ell1 + params.ell2)
    args = (data['pos'], data['los'], data['w'], rand['pos'], rand['los'],
            rand['w'], alpha)
    dn_00 = fourier_transform(_ylm_wgtd_field(*args, 0, 0, params), params)
    N_00 = fourier_transform(_ylm_wgtd_quad_field(*args, 0, 0, params),
                             params)
    win = assignment_window(params)
    alias = shotnoise_aliasing(params)
    win_pk = (win * win) if params.interlace else alias
    kvec = grid_wavevectors(params)
    kmag = vec3_mag(*kvec)
    rvec = grid_positions(params)
    rmag = vec3_mag(*rvec)
    sj_a = SphericalBessel(params.ell1)
    sj_b = SphericalBessel(params.ell2)
    out = _empty_3pcf(ndv)
    for term_idx, (m1, m2, M, coupling) in enumerate(_sph_orders_lpp(params)):
        zero = (m1 == 0 and m2 == 0 and M == 0)
        factor_mirror = 0. if zero else (-1.) ** params.ELL
        factor_mirror_w3j = 0. if zero else 1.
        ylm_r_a = ylm_grid(params.ell1, m1, rvec)
        ylm_r_b = ylm_grid(params.ell2, m2, rvec)
        ylm_k_a = ylm_grid(params.ell1, m1, kvec)
        ylm_k_b = ylm_grid(params.ell2, m2, kvec)
        dn_LM = fourier_transform(
            _ylm_wgtd_field(*args, params.ELL, M, params), params)
        Sbar = shotnoise_amp_bispec(data['los'], data['w'], rand['los'],
                                    rand['w'], alpha, params.ELL, M)
        xi = twopt_field(dn_LM, N_00, Sbar, params, win_pk, alias)
        npairs, r_eff, xi_b = shotnoise_3pcf(xi, ylm_r_a, ylm_r_b, rmag,
                                             edges, centres, params)
        for i, b in _sn_3pcf_diag_entries(params.shape, pairs, len(centres),
                                          params.idx_bin):
            out['sn'][i] += coupling * factor_parity * (
                xi_b[b] + factor_mirror_w3j * np.conj(xi_b[b]))
        _zeta_pairs(out, pairs, centres, npairs, r_eff, term_idx == 0)
        G = inv_fourier_transform(dn_LM / win, params)
        for i in range(ndv):
            Fa = sjl_ylm_ifft(dn_00, ylm_k_a, win, kmag, sj_a,
                              out['r1_eff'][i], params)
            Fb = sjl_ylm_ifft(dn_00, ylm_k_b, win, kmag, sj_b,
                              out['r2_eff'][i], params)
            comp = complex(np.sum(Fa * Fb * G))
            out['zeta'][i] += coupling * params.vol_cell * factor_phase * (
                comp + factor_mirror * np.conj(comp))
    return _finish_3pcf(out, norm_factor)


def _rand_field(rand, alpha_pow, ell, m, params, power=1, conj=False):
    """Single-catalogue ``compute_ylm_wgtd_field`` / ``_quad_field``
    (field.cpp:1325-1362, 1449-1489): the random field times alpha (linear)
    or alpha^2 (quadratic, conjugate Y_lm and w^2)."""
    mr = mesh_weighted(rand['pos'],
                       _ylm_weights(ell, m, rand['los'], rand['w'], power,
                                    conj), params)
    s = alpha_pow * mr.shadow if params.interlace else None
    return Mesh(alpha_pow * mr.field, s)


def wide_angle_pow_law(field, rmag, i_wa, j_wa):
    """``apply_wide_angle_pow_law_kernel`` (field.cpp:1727-1760): times
    r^-(i_wa + j_wa) away from the origin (r >= 1e-6)."""
    far = rmag >= 1.e-6
    out = field.copy()
    out[far] = field[far] * rmag[far] ** (-(i_wa + j_wa))
    return out


def compute_3pcf_window(rand, params, edges, centres, norm_factor,
                        alpha=1., wide_angle=False, i_wa=0, j_wa=0):
    """``trv::compute_3pcf_window`` (threept.cpp:2621-3077): the survey
    3PCF with alpha * (random field) in place of data - alpha * randoms,
    S-bar from the randoms alone (threept.cpp:210-236), and the wide-angle
    kernel on G when requested."""
    _validate_coupling(params)
    pairs = dv_pairs(params.shape, len(centres), params.idx_bin)
    ndv = len(pairs)
    factor_phase = (1j) ** (params.ell1 + params.ell2)
    factor_parity = (-1.) ** (params.ell1 + params.ell2)
    n_00 = fourier_transform(_rand_field(rand, alpha, 0, 0, params), params)
    N_00 = fourier_transform(
        _rand_field(rand, alpha ** 2, 0, 0, params, power=2, conj=True),
        params)
    win = assignment_window(params)
    alias = shotnoise_aliasing(params)
    win_pk = (win * win) if params.interlace else alias
    kvec = grid_wavevectors(params)
    kmag = vec3_mag(*kvec)
    rvec = grid_positions(params)
    rmag = vec3_mag(*rvec)
    sj_a = SphericalBessel(params.ell1)
    sj_b = SphericalBessel(params.ell2)
    out = _empty_3pcf(ndv)
    for term_idx, (m1, m2, M, coupling) in enumerate(_sph_orders_lpp(params)):
        zero = (m1 == 0 and m2 == 0 and M == 0)
        factor_mirror = 0. if zero else (-1.) ** params.ELL
        factor_mirror_w3j = 0. if zero else 1.
        ylm_r_a = ylm_grid(params.ell1, m1, rvec)
        ylm_r_b = ylm_grid(params.ell2, m2, rvec)
        ylm_k_a = ylm_grid(params.ell1, m1, kvec)
        ylm_k_b = ylm_grid(params.ell2, m2, kvec)
        n_LM = fourier_transform(
            _rand_field(rand, alpha, params.ELL, M, params), params)
        Sbar = complex(alpha ** 3 * np.sum(
            reduced_ylm(params.ELL, M, rand['los']) * rand['w'] ** 3))
        xi = twopt_field(n_LM, N_00, Sbar, params, win_pk, alias)
        npairs, r_eff, xi_b = shotnoise_3pcf(xi, ylm_r_a, ylm_r_b, rmag,
                                             edges, centres, params)
        for i, b in _sn_3pcf_diag_entries(params.shape, pairs, len(centres),
                                          params.idx_bin):
            out['sn'][i] += coupling * factor_parity * (
                xi_b[b] + factor_mirror_w3j * np.conj(xi_b[b]))
        _zeta_pairs(out, pairs, centres, npairs, r_eff, term_idx == 0)
        G = inv_fourier_transform(n_LM / win, params)
        if wide_angle:
            G = wide_angle_pow_law(G, rmag, i_wa, j_wa)
        for i in range(ndv):
            Fa = sjl_ylm_ifft(n_00, ylm_k_a, win, kmag, sj_a,
                              out['r1_eff'][i], params)
            Fb = sjl_ylm_ifft(n_00, ylm_k_b, win, kmag, sj_b,
                              out['r2_eff'][i], params)
            comp = complex(np.sum(Fa * Fb * G))
            out['zeta'][i] += coupling * params.vol_cell * factor_phase * (
                comp + factor_mirror * np.conj(comp))
    return _finish_3pcf(out, norm_factor)


def compute_powspec_in_gpp_box(pos, params, edges, centres, norm_factor):
    """``trv::compute_powspec_in_gpp_box`` (twopt.cpp:609-701)."""
    npart = pos.shape[0]
    dn_k = fourier_transform(_unit_mesh_fluct(pos, params), params)
    win = assignment_window(params)
    alias = shotnoise_aliasing(params)
    win_pk = (win * win) if params.interlace else alias
    kvec = grid_wavevectors(params)
    kmag = vec3_mag(*kvec)
    st = twopt_stats_in_fourier(dn_k, dn_k, complex(float(npart)),
                                params.ELL, 0, edges, centres, params, kvec,
                                kmag, win_pk, alias)
    f = float(2 * params.ELL + 1)
    return dict(kbin=np.asarray(centres), keff=st['k'], nmodes=st['nmodes'],
                pk_raw=norm_factor * f * st['pk'],
                pk_shot=norm_factor * f * st['sn'])


def compute_powspec(data, rand, params, edges, centres, norm_factor):
    """``trv::compute_powspec`` (twopt.cpp:388-496)."""
    alpha = float(np.sum(data['ws'])) / float(np.sum(rand['ws']))
    args = (data['pos'], data['los'], data['w'], rand['pos'], rand['los'],
            rand['w'], alpha)
    ell1 = params.ELL
    nb = len(centres)
    dn_00 = fourier_transform(_ylm_wgtd_field(*args, 0, 0, params), params)
    win = assignment_window(params)
    alias = shotnoise_aliasing(params)
    win_pk = (win * win) if params.interlace else alias
    kvec = grid_wavevectors(params)
    kmag = vec3_mag(*kvec)
    nmodes = np.zeros(nb, np.int64)
    keff = np.zeros(nb)
    pk = np.zeros(nb, np.complex128)
    sn = np.zeros(nb, np.complex128)
    for M in range(-params.ELL, params.ELL + 1):
        dn_LM = fourier_transform(
            _ylm_wgtd_field(*args, params.ELL, M, params), params)
        sn_amp = shotnoise_amp_powspec(data['los'], data['w'], rand['los'],
                                       rand['w'], alpha, params.ELL, M)
        for m1 in range(-ell1, ell1 + 1):
            coupling = calc_coupling_coeff_2pt(ell1, params.ELL, m1, M)
            if abs(coupling) < EPS_COUPLING:
                continue
            st = twopt_stats_in_fourier(dn_LM, dn_00, sn_amp, ell1, m1,
                                        edges, centres, params, kvec, kmag,
                                        win_pk, alias)
            pk += coupling * st['pk']
            sn += coupling * st['sn']
            if M == 0 and m1 == 0:
                nmodes = st['nmodes'].copy()
                keff = st['k'].copy()
    return dict(kbin=np.asarray(centres), keff=keff, nmodes=nmodes,
                pk_raw=norm_factor * pk, pk_shot=norm_factor * sn)


# ---------------------------------------------------------------------------
# Normalisation (threept.cpp:96-149, twopt.cpp:56-130, field.cpp:2017-2065)
# ---------------------------------------------------------------------------

def bispec_norm_from_particles(nz, ws, wc, alpha=1.):
    """threept.cpp:96-136: 1 / (alpha sum ws nz^2 wc^3)."""
    norm = float(np.sum(ws * nz ** 2 * wc ** 3))
    if norm == 0.:
        raise ValueError("Particle 'nz' values appear to be all zeros.")
    return 1. / (alpha * norm)


def powspec_norm_from_particles(nz, ws, wc, alpha=1.):
    """twopt.cpp:56-90: 1 / (alpha sum ws nz wc^2)."""
    norm = float(np.sum(ws * nz * wc ** 2))
    if norm == 0.:
        raise ValueError("Particle 'nz' values appear to be all zeros.")
    return 1. / (alpha * norm)


def grid_powlaw_norm(pos, w, params, order):
    """``calc_grid_based_powlaw_norm`` (field.cpp:2017-2065) without
    interlacing: 1 / (dV sum_x Re[n(x)]^order)."""
    p = Params(params.boxsize, params.ngrid, params.assignment, False)
    mesh = assign_weighted_field_to_mesh(pos, w.astype(np.complex128), p)
    return 1. / (float(np.sum(mesh.real ** order)) * p.vol_cell)


# ---------------------------------------------------------------------------
# Catalogue preparation (catalogue.py)
# ---------------------------------------------------------------------------

def periodise(x, y, z, boxsize):
    """``ParticleCatalogue.periodise`` (catalogue.py:648-676)."""
    out = []
    for c, L in zip((x, y, z), boxsize):
        c = np.asarray(c, dtype=np.float64)
        out.append((c + L / 2. - (c.max() + c.min()) / 2.) % L)
    return out


def centre(x, y, z, boxsize, ref=None):
    """``ParticleCatalogue.centre`` (catalogue.py:490-545): shift so that
    the reference catalogue's bounds mid-point is at the box centre."""
    ref = (x, y, z) if ref is None else ref
    origin = [(np.min(r) + np.max(r)) / 2. - L / 2.
              for r, L in zip(ref, boxsize)]
    return [np.asarray(c, dtype=np.float64) - o
            for c, o in zip((x, y, z), origin)], origin


def compute_los(x, y, z):
    """``ParticleCatalogue.compute_los`` (catalogue.py:437-458)."""
    n = np.sqrt(np.asarray(x) ** 2 + np.asarray(y) ** 2
                + np.asarray(z) ** 2)
    n = np.where(n == 0., 1., n)
    return np.stack([x / n, y / n, z / n], axis=-1)


def pad(x, y, z, boxsize, ngrid=None, boxsize_pad=None, ngrid_pad=None,
        ref=None):
    """``ParticleCatalogue.pad`` (catalogue.py:547-646): the reference
    catalogue's minimum moves to boxsize_pad * boxsize, or to
    ngrid_pad * (boxsize / ngrid)."""
    ref = (x, y, z) if ref is None else ref
    origin = np.array([np.min(r) for r in ref])
    if boxsize_pad is not None:
        origin -= np.multiply(boxsize_pad, boxsize)
    if ngrid_pad is not None:
        origin -= np.multiply(ngrid_pad, np.divide(boxsize, ngrid))
    return [np.asarray(c, dtype=np.float64) - o
            for c, o in zip((x, y, z), origin)], origin


def pad_cpp(x, y, z, boxsize, ngrid=None, boxsize_pad=None, ngrid_pad=None,
            ref=None):
    """``ParticleCatalogue::pad_in_box`` / ``pad_grids``
    (particles.cpp:780-888): the same shift with pad_grids' association
    ngrid_pad * boxsize / ngrid, evaluated left to right."""
    ref = (x, y, z) if ref is None else ref
    origin = []
    for a in range(3):
        o = float(np.min(ref[a]))
        if boxsize_pad is not None:
            o = o - boxsize_pad[a] * boxsize[a]
        if ngrid_pad is not None:
            o = o - ngrid_pad[a] * boxsize[a] / float(ngrid[a])
        origin.append(o)
    return [np.asarray(c, dtype=np.float64) - o
            for c, o in zip((x, y, z), origin)], origin


def offset_coords_for_periodicity(x, y, z, boxsize):
    """``ParticleCatalogue::offset_coords_for_periodicity``
    (particles.cpp:678-699): x >= L -> fmod(x, L); x < 0 ->
    fmod(x, L) + L."""
    out = []
    for c, L in zip((x, y, z), boxsize):
        c = np.asarray(c, dtype=np.float64)
        r = c.copy()
        hi, lo = c >= L, c < 0.
        r[hi] = np.fmod(c[hi], L)
        r[lo] = np.fmod(c[lo], L) + L
        out.append(r)
    return out


def load_catalogue_text(paths, columns, volume=0.):
    """``ParticleCatalogue::load_catalogue_file`` for text files
    (particles.cpp:94-510), one Python float per entry: `paths` joined by
    "::", lines that are empty or start with '#' skipped, field f taken
    from the first column named f; absent nz = ntotal / volume (0 if
    volume <= 0), absent ws = wc = 1, w = ws wc."""
    names = columns.split(',')
    fields = ['x', 'y', 'z', 'nz', 'ws', 'wc']
    index = {f: (names.index(f) if f in names else -1) for f in fields}
    rows = []
    for path in [p for p in paths.split('::') if p]:
        with open(path) as fin:
            for line in fin:
                line = line.rstrip('\n')
                if not line.strip() or line.startswith('#'):
                    continue
                rows.append([float(v) for v in line.split()])
    n = len(rows)
    nz_default = n / volume if volume > 0. else 0.
    out = {}
    for f in fields:
        if index[f] >= 0:
            out[f] = np.array([r[index[f]] for r in rows], dtype=np.float64)
        else:
            v = nz_default if f == 'nz' else 1.
            out[f] = np.full(n, v)
    out['w'] = out['ws'] * out['wc']
    return out


# ---------------------------------------------------------------------------
# FFTLog Hankel transform (fftlog.cpp; include/fftlog.hpp:68-257)
# ---------------------------------------------------------------------------

def _lngamma(z):
    from scipy.special import loggamma
    return loggamma(z)


def fftlog_lowring_pivot(mu, q, dL, kr_c=1.):
    """``HankelTransform::calc_lowring_pivot`` (fftlog.cpp:254-295)."""
    y = np.pi / (2. * dL)
    if kr_c > 0.:
        gp = _lngamma(complex((mu + 1. + q) / 2., y))
        gm = _lngamma(complex((mu + 1. - q) / 2., y))
        argphase = np.log(2. / kr_c) / dL + (gp.imag + gm.imag) / np.pi
        return kr_c * np.exp(dL * (argphase - np.round(argphase)))
    nu = complex(q, 2. * y)
    lr = _lngamma((mu + 1. + nu) / 2.) - _lngamma((mu + 1. - nu) / 2.)
    lnkr = np.log(2.) + lr.imag / (2. * y)
    return np.exp(lnkr - np.floor(lnkr / dL) * dL)


def fftlog_kernel(mu, q, N, dL, kr_c):
    """``HankelTransform::compute_kernel_coeff`` (fftlog.cpp:297-356)."""
    y = np.pi / (N * dL)
    t = -2. * y * np.log(kr_c / 2.)
    m = np.arange(N // 2 + 1)
    if q == 0.:
        ge = _lngamma((mu + 1.) / 2. + 1j * m * y)
        half = np.exp(1j * (m * t + 2. * ge.imag))
    else:
        gp = _lngamma((mu + 1. + q) / 2. + 1j * m * y)
        gm = _lngamma((mu + 1. - q) / 2. + 1j * m * y)
        half = np.exp(q * np.log(2.) + gp.real - gm.real) \
            * np.exp(1j * (m * t + gp.imag + gm.imag))
    u = np.empty(N, dtype=complex)
    u[:N // 2 + 1] = half
    u[N // 2 + 1:] = np.conj(half[1:N - N // 2][::-1])
    if N % 2 == 0:
        u[N // 2] = u[N // 2].real
    return u


def _extend_native(a, n_ext, option):
    """``extrap_pad`` / ``extrap_lin`` / ``extrap_loglin``
    (arrayops.cpp:94-203) on a real row."""
    left_i = np.arange(-n_ext, 0)
    right_i = np.arange(1, n_ext + 1)
    if option == 1:
        lo, hi = np.zeros(n_ext), np.zeros(n_ext)
    elif option == 2:
        lo, hi = np.full(n_ext, a[0]), np.full(n_ext, a[-1])
    elif option == 3:
        lo = a[0] + left_i * (a[1] - a[0])
        hi = a[-1] + right_i * (a[-1] - a[-2])
    else:
        lo = a[0] * np.exp(left_i * np.log(a[1] / a[0]))
        hi = a[-1] * np.exp(right_i * np.log(a[-1] / a[-2]))
    return np.concatenate([lo, a, hi])


def hankel_transform(mu, q, x, a, kr_c=1., lowring=True, extrap=0,
                     extrap_exp=2.):
    """``HankelTransform::initialise`` + ``biased_transform``
    (fftlog.cpp:108-252, 358-478): post-transform points and samples."""
    x = np.asarray(x, dtype=float)
    N = len(x)
    dL = np.log(x[-1] / x[0]) / (N - 1)
    if extrap:
        Nt = int(2 ** np.ceil(np.log2(extrap_exp * N)))
        n_ext = (Nt - N) // 2
    else:
        Nt, n_ext = N, 0
    piv = fftlog_lowring_pivot(mu, q, dL, kr_c) if lowring else kr_c
    u = fftlog_kernel(mu, q, Nt, dL, piv)
    post = piv * np.exp(-dL) / x[::-1]
    if extrap:
        pre = _extend_native(np.real(np.asarray(a)), n_ext, extrap)
    else:
        pre = np.asarray(a, dtype=complex)
    b = np.fft.fft(np.fft.fft(pre) * u / Nt)
    return post, b[n_ext:n_ext + N]
