"""Allocation-free grid-based normalisation against the context entry point.

Collected last on purpose: it must give the same answers in a fresh
process (its first call does the per-device set-up) and after every other
GPU test has run on the same device.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from triumvirate_gb300 import _engine, _lib  # noqa: E402

# FP64 atomics deposit in a different order in the two entry points.
RTOL = 1e-12


def _params(box, ngrid, order):
    return _engine.make_params(
        {'boxsize': dict(zip('xyz', box)), 'ngrid': dict(zip('xyz', ngrid)),
         'assignment_order': order, 'interlace': False, 'degrees': {},
         'form': 'diag', 'precision': 'fp64', 'verbose': 0}, '2pt')


def _device_catalogue(n, box, seed, weighted):
    rng = np.random.default_rng(seed)
    cols = [torch.from_numpy(rng.uniform(0., b, n)).cuda() for b in box]
    if weighted:
        cols.append(torch.from_numpy(rng.uniform(0.5, 1.5, n)).cuda())
    torch.cuda.synchronize()
    ptrs = [t.data_ptr() for t in cols]
    cat = _engine.device_catalogue(n, *ptrs[:3],
                                   w_ptr=ptrs[3] if weighted else None)
    return cat, cols


def _noalloc(pc, cat, power):
    out = C.c_double()
    stream = torch.cuda.current_stream().cuda_stream
    _lib.check(_lib.load().trvg_calc_grid_based_powlaw_norm_noalloc(
        C.byref(pc), C.byref(cat), int(power), C.c_void_p(stream),
        C.byref(out)))
    return out.value


@pytest.mark.parametrize("box, ngrid, order, power, n, weighted", [
    ((1000., 1000., 1000.), (64, 64, 64), 3, 2, 200_000, True),
    ((600., 700., 800.), (48, 40, 56), 4, 3, 50_000, False),
    ((500., 500., 500.), (128, 128, 128), 2, 2, 300_000, True),
])
def test_noalloc_matches_context_entry(box, ngrid, order, power, n, weighted):
    torch.cuda.set_device(0)
    pc = _params(box, ngrid, order)
    cat, keep = _device_catalogue(n, box, 7, weighted)
    ref = _engine.grid_powlaw_norm(_lib.default_context(), pc, cat, power)
    first = _noalloc(pc, cat, power)
    second = _noalloc(pc, cat, power)
    for got in (first, second):
        assert abs(got / ref - 1.) < RTOL, (got, ref)
    del keep


def test_noalloc_rejects_oversized_mesh_and_host_arrays():
    pc = _params((1000.,) * 3, (256, 128, 128), 3)
    cat, keep = _device_catalogue(1000, (1000.,) * 3, 1, False)
    with pytest.raises(_lib.InvalidParameterError, match="static scratch"):
        _noalloc(pc, cat, 2)
    host = _engine.HostCatalogue(*(np.full(10, 1.) for _ in range(3)))
    with pytest.raises(_lib.InvalidParameterError, match="device-resident"):
        _noalloc(_params((1000.,) * 3, (32, 32, 32), 3), host.c, 2)
    del keep
