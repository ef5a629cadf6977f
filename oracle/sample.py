"""Timing harness of the oracle on the periodic-box bispectrum workload.

TEST INFRASTRUCTURE ONLY (the CPU baseline of ``bench.py``).  It runs the
oracle's restatement of ``trv::compute_bispec_in_gpp_box``
(threept.cpp:1473-2188) in the reference's own order of work, split into
the per-estimate set-up and the per-bin-pair unit that the reference
repeats for every pair:

* set-up: assignment + FFT of delta n_00, of N_L0 and of G_00, the
  compensation and inverse FFT of G_00 (threept.cpp:1552-1670);
* pair: two band-limited inverse FFTs, the triple-product reduction, the
  shot-noise inverse FFT and its spline-weighted reduction
  (threept.cpp:1675-1723, 2126-2140).

The set-up also forms the fine-binned two-point statistics of the
single-leg shot-noise terms (threept.cpp:1974-2060), so that ``entry``
returns the oracle's normalised bk_raw, bk_shot and mode count of one
diagonal bin: the check of the GPU estimate at the full workload size.
"""
from __future__ import annotations

import os

import numpy as np

from . import trv_oracle as O


class GppBispecSample:
    """Oracle B_000 diag estimate split into set-up and bin pairs."""

    def __init__(self, npart, boxsize, ngrid, nbins, seed=42):
        self.threads = os.cpu_count() or 1
        rng = np.random.default_rng(seed)
        x, y, z = rng.uniform(0., boxsize, size=(3, npart))
        self.pos = np.stack(O.periodise(x, y, z, [boxsize] * 3), -1)
        self.p = O.Params(boxsize, ngrid, 'tsc', False, 0, 0, 0)
        self.edges, self.centres = O.lin_binning(0.005, 0.205, nbins)
        self.npart = npart

    def setup(self):
        p = self.p
        self.dn_k = O.fourier_transform(O._unit_mesh_fluct(self.pos, p), p)
        self.N_k = O.fourier_transform(O._unit_mesh(self.pos, p), p)
        g_k = O.fourier_transform(O._unit_mesh_fluct(self.pos, p), p)
        self.win = O.assignment_window(p)
        self.alias = O.shotnoise_aliasing(p)
        self.G = O.inv_fourier_transform(g_k / self.win, p)
        del g_k
        self.kmag = O.vec3_mag(*O.grid_wavevectors(p))
        self.rmag = O.vec3_mag(*O.grid_positions(p))
        self.ones = np.ones(self.kmag.shape, dtype=np.complex128)
        self.sj = O.SphericalBessel(0)
        # Single-leg shot-noise terms S_i_jk = S_ik_j (ell1 = ell2 = 0).
        win_pk = self.alias
        st = O.twopt_stats_in_fourier(
            self.dn_k, self.N_k, complex(float(self.npart)), 0, 0,
            self.edges, self.centres, p, O.grid_wavevectors(p), self.kmag,
            win_pk, self.alias)
        self.S_leg = st['pk'] - st['sn']

    def pair(self, b):
        p = self.p
        lo, hi = self.edges[b], self.edges[b + 1]
        Fa, keff, nm = O.band_limited_ifft(self.dn_k, self.ones, self.win,
                                           self.kmag, lo, hi)
        Fb, _, _ = O.band_limited_ifft(self.dn_k, self.ones, self.win,
                                       self.kmag, lo, hi)
        comp = complex(np.sum(Fa * Fb * self.G))
        del Fa, Fb
        xi = O.twopt_field(self.dn_k, self.N_k, complex(float(self.npart)), p,
                           self.alias, self.alias)
        s = O.shotnoise_bispec_per_bin(xi, 1., 1., self.sj, self.sj,
                                       self.rmag, keff, keff, p)
        self.last = (b, comp, s, nm)
        return comp, s

    def entry(self, b, norm):
        """bk_raw, bk_shot and nmodes of diagonal entry (b, b) of B_000
        (coupling 1, no mirror term; threept.cpp:1703-1723, 1974-2140),
        from the last ``pair(b)``."""
        if getattr(self, 'last', (None,))[0] != b:
            self.pair(b)
        _, comp, s, nm = self.last
        raw = norm * self.p.vol_cell * comp
        shot = norm * (complex(float(self.npart)) + 2. * self.S_leg[b] + s)
        return raw, shot, nm
