"""Allocation-free grid-based normalisation against the context entry point.

Collected last on purpose: it must give the same answers after every other
GPU test has run on the same device, and in a fresh process where it is
the first call into the library (that call does the per-device set-up);
`test_noalloc_first_call_in_fresh_process` runs that case in a child
process.
"""
import ctypes as C
import json
import os
import subprocess
import sys
import textwrap
from pathlib import Path

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


_FRESH = textwrap.dedent("""
    import ctypes as C, json, sys
    import numpy as np, torch
    sys.path.insert(0, sys.argv[1])
    from triumvirate_gb300 import _engine, _lib
    torch.cuda.set_device(0)
    box, ngrid, n = (800., 800., 800.), (64, 64, 64), 100_000
    rng = np.random.default_rng(3)
    cols = [torch.from_numpy(rng.uniform(0., b, n)).cuda() for b in box]
    torch.cuda.synchronize()
    cat = _engine.device_catalogue(n, *[t.data_ptr() for t in cols])
    pc = _engine.make_params(
        {'boxsize': dict(zip('xyz', box)), 'ngrid': dict(zip('xyz', ngrid)),
         'assignment_order': 3, 'interlace': False, 'degrees': {},
         'form': 'diag', 'precision': 'fp64', 'verbose': 0}, '2pt')
    fn = _lib.load().trvg_calc_grid_based_powlaw_norm_noalloc
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    out, free = [], []
    for _ in range(2):
        v = C.c_double()
        _lib.check(fn(C.byref(pc), C.byref(cat), 2, stream, C.byref(v)))
        out.append(v.value)
        free.append(torch.cuda.mem_get_info()[0])
    ref = _engine.grid_powlaw_norm(_lib.default_context(), pc, cat, 2)
    print(json.dumps({"noalloc": out, "ref": ref, "free": free}))
""")


def test_noalloc_first_call_in_fresh_process():
    """The entry point as the first library call of a process: the
    per-device set-up runs inside it, both calls match the context entry
    point made afterwards, and the second call leaves free device memory
    unchanged."""
    root = Path(__file__).resolve().parents[1]
    r = subprocess.run([sys.executable, "-c", _FRESH, str(root)],
                       capture_output=True, text=True, timeout=600,
                       env=dict(os.environ))
    assert r.returncode == 0, r.stderr[-2000:]
    got = json.loads(r.stdout.strip().splitlines()[-1])
    for v in got["noalloc"]:
        assert abs(v / got["ref"] - 1.) < RTOL, got
    assert got["free"][0] == got["free"][1], got
