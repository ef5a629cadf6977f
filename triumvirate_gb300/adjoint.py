"""Gradients of the periodic-box bispectrum B_000 (the reference library
has no derivatives).

``bispec_gpp_vjp`` returns dL/d(mesh), dL/d(weights) and dL/d(positions)
for cotangents dL/dB of the raw data vector and of its shot noise;
``bispec_gpp`` wraps the forward estimate and the adjoint in a
``torch.autograd.Function`` of particle positions and weights (B = raw -
shot by default), and ``bispec_gpp_mesh`` in one of a count mesh (raw B of
the mesh's fluctuation about its mean).  They call ``trvg_bispec_gpp_vjp``,
which recomputes the shell fields instead of storing them from the
forward pass; ``bispec_gpp_adjoint`` is the raw part for particles.

Positions must already lie in [0, L) (the box is not periodised here).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _engine, _lib

_ORDERS = {'ngp': 1, 'cic': 2, 'tsc': 3, 'pcs': 4}


class BispecGppConfig:
    """Sampling and binning of a differentiable B_000 estimate."""

    def __init__(self, boxsize, ngrid, binning, assignment='tsc',
                 form='diag', idx_bin=0, precision='fp32mixed', norm=None,
                 device=0):
        box = np.broadcast_to(np.asarray(boxsize, dtype=float), 3)
        grid = np.broadcast_to(np.asarray(ngrid, dtype=int), 3)
        self.boxsize = [float(b) for b in box]
        self.ngrid = [int(n) for n in grid]
        self.binning = binning
        self.shape = form
        self.idx_bin = int(idx_bin or 0)
        self.norm = norm
        self.params = _engine.make_params(
            {'boxsize': dict(zip('xyz', self.boxsize)),
             'ngrid': dict(zip('xyz', self.ngrid)),
             'assignment_order': _ORDERS[assignment], 'interlace': False,
             'degrees': {'ell1': 0, 'ell2': 0, 'ELL': 0}, 'form': form,
             'shape': form, 'idx_bin': self.idx_bin, 'precision': precision,
             'verbose': 0}, '3pt')
        self.ctx = _lib.default_context(device)
        self.dim = _engine.dv_dim(form, binning.num_bins, self.idx_bin)

    def norm_for(self, n):
        """Particle normalisation 1 / (N nbar^2) of N unit-weight particles
        at nbar = N / V, unless a norm was given."""
        if self.norm is not None:
            return float(self.norm)
        vol = float(np.prod(self.boxsize))
        return 1. / (n * (n / vol) ** 2)


def _columns(torch, positions, weights):
    x, y, z = (positions[:, a].contiguous() for a in range(3))
    w = None if weights is None else weights.contiguous()
    return x, y, z, w


def _catalogue(x, y, z, w):
    return _engine.device_catalogue(
        x.numel(), x.data_ptr(), y.data_ptr(), z.data_ptr(),
        None if w is None else w.data_ptr())


def bispec_gpp_adjoint(positions, weights, cotangent, cfg, mesh=False):
    """dL/dm, dL/dw and dL/dx for L with dL/d(raw B) = `cotangent`.

    `positions` (n, 3) and `weights` (n,) or None are float64 CUDA
    tensors; returns a dict with 'raw' (the forward raw values, complex
    numpy), 'grad_w' (n,), 'grad_pos' (n, 3) and, if `mesh`, 'grad_mesh'
    (ngrid[0], ngrid[1], ngrid[2]) tensors on the same device.
    """
    import torch
    x, y, z, w = _columns(torch, positions, weights)
    n = x.numel()
    cat = _catalogue(x, y, z, w)
    cot = np.zeros(2 * cfg.dim)
    cot[0::2] = np.asarray(cotangent, dtype=np.float64).reshape(-1)
    gw = torch.empty(n, dtype=torch.float64, device=x.device)
    gp = torch.empty(3 * n, dtype=torch.float64, device=x.device)
    gm = (torch.empty(int(np.prod(cfg.ngrid)), dtype=torch.float64,
                      device=x.device) if mesh else None)
    res = _engine.ThreeptResult(cfg.dim)
    hb = _engine.HostBinning(cfg.binning)
    torch.cuda.synchronize(x.device)
    _lib.check(_lib.load().trvg_bispec_gpp_adjoint(
        cfg.ctx.handle, C.byref(cfg.params), C.byref(cat), C.byref(hb.c),
        cfg.norm_for(n), _lib.dptr(cot),
        None if gm is None else gm.data_ptr(), gw.data_ptr(), gp.data_ptr(),
        C.byref(res.c)))
    out = {'raw': res.as_dict('bispec')['bk_raw'], 'grad_w': gw,
           'grad_pos': gp.reshape(3, n).t().contiguous()}
    if gm is not None:
        out['grad_mesh'] = gm.reshape(cfg.ngrid)
    return out


def bispec_gpp_vjp(cfg, cot_raw, cot_shot=None, positions=None,
                   weights=None, mesh=None, want_mesh=False):
    """Vector-Jacobian product of raw B_000 and its shot noise.

    Give `positions` (n, 3) and `weights` (n,) or None (float64 CUDA
    tensors), or a count `mesh` (float32 CUDA tensor of shape ngrid: the
    weight deposited per cell).  `cot_raw` and `cot_shot` are dL/d(real
    part) per data-vector entry (cot_shot: particles only).  Returns a dict
    with 'raw' (the forward raw values, complex numpy) and 'grad_mesh' (if
    `want_mesh` or a mesh was given), 'grad_w', 'grad_pos' (particles)."""
    import torch
    lib = _lib.load()
    cr = np.zeros(2 * cfg.dim)
    cr[0::2] = np.asarray(cot_raw, dtype=np.float64).reshape(-1)
    cs = None
    if cot_shot is not None:
        cs = np.zeros(2 * cfg.dim)
        cs[0::2] = np.asarray(cot_shot, dtype=np.float64).reshape(-1)
    res = _engine.ThreeptResult(cfg.dim)
    hb = _engine.HostBinning(cfg.binning)
    out = {}
    if mesh is not None:
        m = mesh.detach().to(torch.float32).contiguous()
        gm = torch.empty(int(np.prod(cfg.ngrid)), dtype=torch.float64,
                         device=m.device)
        torch.cuda.synchronize(m.device)
        _lib.check(lib.trvg_bispec_gpp_vjp(
            cfg.ctx.handle, C.byref(cfg.params), None, m.data_ptr(),
            C.byref(hb.c), float(cfg.norm if cfg.norm is not None else 1.),
            _lib.dptr(cr), None, gm.data_ptr(), None, None, C.byref(res.c)))
        torch.cuda.synchronize(m.device)
        out['grad_mesh'] = gm.reshape(cfg.ngrid)
    else:
        x, y, z, w = _columns(torch, positions, weights)
        n = x.numel()
        cat = _catalogue(x, y, z, w)
        gw = torch.empty(n, dtype=torch.float64, device=x.device)
        gp = torch.empty(3 * n, dtype=torch.float64, device=x.device)
        gm = (torch.empty(int(np.prod(cfg.ngrid)), dtype=torch.float64,
                          device=x.device) if want_mesh else None)
        torch.cuda.synchronize(x.device)
        _lib.check(lib.trvg_bispec_gpp_vjp(
            cfg.ctx.handle, C.byref(cfg.params), C.byref(cat), None,
            C.byref(hb.c), cfg.norm_for(n), _lib.dptr(cr),
            None if cs is None else _lib.dptr(cs),
            None if gm is None else gm.data_ptr(), gw.data_ptr(),
            gp.data_ptr(), C.byref(res.c)))
        torch.cuda.synchronize(x.device)
        out['grad_w'] = gw
        out['grad_pos'] = gp.reshape(3, n).t().contiguous()
        if gm is not None:
            out['grad_mesh'] = gm.reshape(cfg.ngrid)
    out['raw'] = res.as_dict('bispec')['bk_raw']
    return out


def _forward(positions, weights, cfg):
    import torch
    x, y, z, w = _columns(torch, positions, weights)
    torch.cuda.synchronize(x.device)
    res = _engine.call_threept(
        'trvg_compute_bispec_in_gpp_box', cfg.ctx, cfg.params,
        _catalogue(x, y, z, w), cfg.binning, cfg.norm_for(x.numel()),
        'bispec', shape=cfg.shape, idx_bin=cfg.idx_bin)
    return res


def bispec_gpp(positions, weights, cfg, shot_noise=True):
    """Real part of B_000 = raw - shot (raw alone with shot_noise=False)
    per data-vector entry as a differentiable function of `positions`
    (n, 3) and `weights` (n,) or None (float64, CUDA)."""
    import torch

    class _Bispec(torch.autograd.Function):
        @staticmethod
        def forward(ctx, pos, wts):
            res = _forward(pos, wts, cfg)
            ctx.save_for_backward(pos, wts)
            b = res['bk_raw'] - (res['bk_shot'] if shot_noise else 0.)
            return torch.as_tensor(np.ascontiguousarray(b.real),
                                   device=pos.device)

        @staticmethod
        def backward(ctx, grad_out):
            pos, wts = ctx.saved_tensors
            lam = grad_out.detach().cpu().numpy()
            g = bispec_gpp_vjp(cfg, lam, -lam if shot_noise else None,
                               positions=pos, weights=wts)
            # No gradient flows to an absent weight column.
            return g['grad_pos'], (g['grad_w'] if wts is not None else None)

    return _Bispec.apply(positions, weights)


def bispec_gpp_mesh(mesh, cfg):
    """Real part of raw B_000 per data-vector entry as a differentiable
    function of a count mesh (float32 CUDA tensor of shape ngrid, the
    weight per cell; its fluctuation is taken about its own mean).  The
    normalisation is cfg.norm (1 if unset)."""
    import torch

    class _BispecMesh(torch.autograd.Function):
        @staticmethod
        def forward(ctx, m):
            g = bispec_gpp_vjp(cfg, np.zeros(cfg.dim), mesh=m)
            ctx.save_for_backward(m)
            return torch.as_tensor(np.ascontiguousarray(g['raw'].real),
                                   device=m.device)

        @staticmethod
        def backward(ctx, grad_out):
            (m,) = ctx.saved_tensors
            g = bispec_gpp_vjp(cfg, grad_out.detach().cpu().numpy(), mesh=m)
            return g['grad_mesh'].to(m.dtype)

    return _BispecMesh.apply(mesh)
