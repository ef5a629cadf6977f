"""ctypes bindings of ``libtrvg.so`` (declared in ``include/trvg.h``).

The library is built in the source tree by ``triumvirate_gb300.build``.  No
computation falls back to the CPU: if the library cannot be loaded, every
estimator raises.
"""
from __future__ import annotations

import ctypes as C
import os
import threading
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "libtrvg.so"

TRVG_OK = 0
TRVG_ERR_INVALID_PARAMETER = 1
TRVG_ERR_INVALID_DATA = 2
TRVG_ERR_UNIMPLEMENTED = 3
TRVG_ERR_CUDA = 4
TRVG_ERR_CUFFT = 5
TRVG_ERR_ALLOC = 6

SHAPES = {'diag': 0, 'off-diag': 1, 'row': 2, 'full': 3, 'triu': 4}
PRECISIONS = {'fp64': 0, 'fp32mixed': 1}
MEM_HOST, MEM_DEVICE = 0, 1

EXPORTED = [
    "trvg_context_create", "trvg_context_destroy", "trvg_last_error",
    "trvg_version", "trvg_get_stats", "trvg_release_workspace",
    "trvg_data_vector_dim",
    "trvg_compute_bispec_in_gpp_box", "trvg_compute_bispec",
    "trvg_compute_3pcf_in_gpp_box", "trvg_compute_3pcf",
    "trvg_compute_powspec_in_gpp_box", "trvg_compute_powspec",
    "trvg_calc_grid_based_powlaw_norm", "trvg_assign_weighted_field_to_mesh",
    "trvg_wigner_3j", "trvg_sph_bessel", "trvg_sph_bessel_spline",
    "trvg_reduced_ylm", "trvg_context_set_stream", "trvg_set_option",
    "trvg_kernel_time_count", "trvg_kernel_time_get",
    "trvg_calc_grid_based_powlaw_norm_noalloc",
    "trvg_compute_bispec_in_gpp_box_batch", "trvg_bispec_gpp_adjoint",
    "trvg_bispec_gpp_vjp",
    "trvg_compute_3pcf_window", "trvg_tuned_count", "trvg_tuned_get",
    "trvg_hankel_create", "trvg_hankel_info", "trvg_hankel_transform",
    "trvg_hankel_destroy",
    "trvg_dcat_read_text", "trvg_dcat_from_host", "trvg_dcat_info",
    "trvg_dcat_offset", "trvg_dcat_centre", "trvg_dcat_pad",
    "trvg_dcat_wrap_box", "trvg_dcat_periodise", "trvg_dcat_compute_los",
    "trvg_dcat_set_column", "trvg_dcat_upload", "trvg_dcat_norm_sum",
    "trvg_dcat_view", "trvg_dcat_download", "trvg_dcat_destroy",
    "trvg_dcat_concat",
]


class InvalidParameterError(ValueError):
    """``trv::sys::InvalidParameterError`` (monitor.hpp:683-780)."""


class InvalidDataError(RuntimeError):
    """``trv::sys::InvalidDataError``."""


class UnimplementedError(NotImplementedError):
    """``trv::sys::UnimplementedError``."""


class DeviceError(RuntimeError):
    """CUDA / cuFFT failure or device allocation failure."""


_ERRORS = {
    TRVG_ERR_INVALID_PARAMETER: InvalidParameterError,
    TRVG_ERR_INVALID_DATA: InvalidDataError,
    TRVG_ERR_UNIMPLEMENTED: UnimplementedError,
    TRVG_ERR_CUDA: DeviceError,
    TRVG_ERR_CUFFT: DeviceError,
    TRVG_ERR_ALLOC: DeviceError,
}


class Params(C.Structure):
    _fields_ = [
        ("boxsize", C.c_double * 3),
        ("ngrid", C.c_int * 3),
        ("assignment_order", C.c_int),
        ("interlace", C.c_int),
        ("ell1", C.c_int), ("ell2", C.c_int), ("ELL", C.c_int),
        ("shape", C.c_int),
        ("idx_bin", C.c_int),
        ("precision", C.c_int),
        ("verbose", C.c_int),
        ("i_wa", C.c_int), ("j_wa", C.c_int),
    ]


class BinningC(C.Structure):
    _fields_ = [
        ("num_bins", C.c_int),
        ("bin_edges", C.POINTER(C.c_double)),
        ("bin_centres", C.POINTER(C.c_double)),
    ]


class Catalogue(C.Structure):
    _fields_ = [
        ("n", C.c_int64),
        ("x", C.c_void_p), ("y", C.c_void_p), ("z", C.c_void_p),
        ("w", C.c_void_p),
        ("los_x", C.c_void_p), ("los_y", C.c_void_p), ("los_z", C.c_void_p),
        ("memory", C.c_int),
    ]


class ThreeptOut(C.Structure):
    _fields_ = [
        ("dim", C.c_int),
        ("coord1_bin", C.POINTER(C.c_double)),
        ("coord1_eff", C.POINTER(C.c_double)),
        ("count_1", C.POINTER(C.c_int32)),
        ("coord2_bin", C.POINTER(C.c_double)),
        ("coord2_eff", C.POINTER(C.c_double)),
        ("count_2", C.POINTER(C.c_int32)),
        ("raw", C.POINTER(C.c_double)),
        ("shot", C.POINTER(C.c_double)),
    ]


class PowspecOut(C.Structure):
    _fields_ = [
        ("dim", C.c_int),
        ("kbin", C.POINTER(C.c_double)),
        ("keff", C.POINTER(C.c_double)),
        ("nmodes", C.POINTER(C.c_int32)),
        ("pk_raw", C.POINTER(C.c_double)),
        ("pk_shot", C.POINTER(C.c_double)),
    ]


class Stats(C.Structure):
    _fields_ = [
        ("ms_total", C.c_double),
        ("ms_h2d", C.c_double),
        ("h2d_bytes", C.c_int64),
        ("kernel_launches", C.c_int64),
        ("fft_launches", C.c_int64),
        ("pruned_grid", C.c_int * 3),
        ("graph_replays", C.c_int64),
    ]


_lib = None
_lib_lock = threading.Lock()


def load(path: str | os.PathLike | None = None):
    """Load the library (once); raise if it is missing."""
    global _lib
    with _lib_lock:
        if _lib is not None:
            return _lib
        p = Path(path) if path else LIB_PATH
        if not p.exists():
            raise ImportError(
                f"{p} is missing: build it with "
                "`python -m triumvirate_gb300.build` (no CPU fallback).")
        lib = C.CDLL(str(p))
        _declare(lib)
        _lib = lib
        return lib


def _declare(lib):
    vp, ip, dp = C.c_void_p, C.c_int, C.c_double
    P = C.POINTER
    lib.trvg_context_create.argtypes = [ip, P(vp)]
    lib.trvg_context_destroy.argtypes = [vp]
    lib.trvg_last_error.restype = C.c_char_p
    lib.trvg_version.restype = C.c_char_p
    lib.trvg_get_stats.argtypes = [vp, P(Stats)]
    lib.trvg_release_workspace.argtypes = [vp]
    lib.trvg_data_vector_dim.argtypes = [ip, ip, ip, P(ip)]
    for nm in ("trvg_compute_bispec_in_gpp_box",
               "trvg_compute_3pcf_in_gpp_box"):
        getattr(lib, nm).argtypes = [vp, P(Params), P(Catalogue),
                                     P(BinningC), dp, P(ThreeptOut)]
    for nm in ("trvg_compute_bispec", "trvg_compute_3pcf"):
        getattr(lib, nm).argtypes = [vp, P(Params), P(Catalogue),
                                     P(Catalogue), dp, P(BinningC), dp,
                                     P(ThreeptOut)]
    lib.trvg_compute_3pcf_window.argtypes = [
        vp, P(Params), P(Catalogue), dp, P(BinningC), dp, ip, P(ThreeptOut)]
    lib.trvg_compute_powspec_in_gpp_box.argtypes = [
        vp, P(Params), P(Catalogue), P(BinningC), dp, P(PowspecOut)]
    lib.trvg_compute_powspec.argtypes = [
        vp, P(Params), P(Catalogue), P(Catalogue), dp, P(BinningC), dp,
        P(PowspecOut)]
    lib.trvg_calc_grid_based_powlaw_norm.argtypes = [
        vp, P(Params), P(Catalogue), ip, P(dp)]
    lib.trvg_assign_weighted_field_to_mesh.argtypes = [
        vp, P(Params), P(Catalogue), ip, P(dp)]
    lib.trvg_compute_bispec_in_gpp_box_batch.argtypes = [
        vp, P(Params), P(Catalogue), ip, P(C.c_int64), P(BinningC), P(dp),
        P(ThreeptOut)]
    lib.trvg_bispec_gpp_adjoint.argtypes = [
        vp, P(Params), P(Catalogue), P(BinningC), dp, P(dp), vp, vp, vp,
        P(ThreeptOut)]
    lib.trvg_bispec_gpp_vjp.argtypes = [
        vp, P(Params), P(Catalogue), vp, P(BinningC), dp, P(dp), P(dp), vp,
        vp, vp, P(ThreeptOut)]
    lib.trvg_calc_grid_based_powlaw_norm_noalloc.argtypes = [
        P(Params), P(Catalogue), ip, vp, P(dp)]
    lib.trvg_wigner_3j.argtypes = [ip] * 6
    lib.trvg_wigner_3j.restype = dp
    lib.trvg_sph_bessel.argtypes = [ip, dp]
    lib.trvg_sph_bessel.restype = dp
    lib.trvg_sph_bessel_spline.argtypes = [ip, P(dp), C.c_int64, P(dp)]
    lib.trvg_reduced_ylm.argtypes = [ip, ip, P(dp), C.c_int64, P(dp)]
    lib.trvg_context_set_stream.argtypes = [vp, vp]
    lib.trvg_set_option.argtypes = [vp, C.c_char_p, C.c_int64]
    lib.trvg_hankel_create.argtypes = [dp, dp, P(dp), ip, dp, ip, ip, dp,
                                       P(vp)]
    lib.trvg_hankel_info.argtypes = [vp, P(ip), P(ip), P(dp), P(dp), P(dp),
                                     P(dp)]
    lib.trvg_hankel_transform.argtypes = [vp, vp, ip, P(dp), P(dp)]
    lib.trvg_hankel_destroy.argtypes = [vp]
    lib.trvg_tuned_count.argtypes = [vp, P(ip)]
    lib.trvg_tuned_get.argtypes = [vp, ip, C.c_char_p, ip, P(C.c_int64)]
    lib.trvg_kernel_time_count.argtypes = [vp, P(ip)]
    lib.trvg_kernel_time_get.argtypes = [vp, ip, C.c_char_p, ip, P(dp),
                                         P(C.c_int64)]
    i64, cp = C.c_int64, C.c_char_p
    lib.trvg_dcat_read_text.argtypes = [vp, cp, cp, dp, P(vp)]
    lib.trvg_dcat_from_host.argtypes = [vp, i64] + [P(dp)] * 6 + [P(vp)]
    lib.trvg_dcat_info.argtypes = [vp, vp, P(i64), P(dp), P(dp), P(dp),
                                   P(dp)]
    lib.trvg_dcat_offset.argtypes = [vp, vp, P(dp)]
    lib.trvg_dcat_centre.argtypes = [vp, vp, vp, P(dp)]
    lib.trvg_dcat_pad.argtypes = [vp, vp, vp, P(dp), P(dp), P(dp), P(dp)]
    lib.trvg_dcat_wrap_box.argtypes = [vp, vp, P(dp)]
    lib.trvg_dcat_periodise.argtypes = [vp, vp, P(dp)]
    lib.trvg_dcat_compute_los.argtypes = [vp, vp]
    lib.trvg_dcat_set_column.argtypes = [vp, vp, cp, dp]
    lib.trvg_dcat_upload.argtypes = [vp, vp, cp, P(dp)]
    lib.trvg_dcat_norm_sum.argtypes = [vp, vp, ip, P(dp), P(i64)]
    lib.trvg_dcat_view.argtypes = [vp, P(Catalogue)]
    lib.trvg_dcat_download.argtypes = [vp, vp, cp, P(dp)]
    lib.trvg_dcat_destroy.argtypes = [vp]
    lib.trvg_dcat_concat.argtypes = [vp, P(vp), ip, P(vp)]


def check(status: int):
    """Raise the Python exception matching a TRVG_* status."""
    if status == TRVG_OK:
        return
    msg = load().trvg_last_error().decode(errors='replace')
    raise _ERRORS.get(status, RuntimeError)(msg or f"trvg status {status}")


def dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def iptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


class Context:
    """A device context: one CUDA stream, FFT plans and cached workspace."""

    def __init__(self, device: int = 0):
        lib = load()
        h = C.c_void_p()
        check(lib.trvg_context_create(int(device), C.byref(h)))
        self._h = h
        self.device = device

    @property
    def handle(self):
        return self._h

    def stats(self) -> dict:
        s = Stats()
        check(load().trvg_get_stats(self._h, C.byref(s)))
        return dict(ms_total=s.ms_total, ms_h2d=s.ms_h2d,
                    h2d_bytes=s.h2d_bytes, kernel_launches=s.kernel_launches,
                    fft_launches=s.fft_launches,
                    pruned_grid=tuple(s.pruned_grid),
                    graph_replays=s.graph_replays)

    def set_stream(self, stream_ptr):
        """Run on a caller's cudaStream_t (None: the context's own)."""
        check(load().trvg_context_set_stream(
            self._h, None if stream_ptr is None else C.c_void_p(stream_ptr)))

    def set_option(self, key: str, value: int):
        check(load().trvg_set_option(self._h, key.encode(), int(value)))

    def kernel_times(self) -> dict:
        """{name: (ms, launches)} of the last call (profiling on)."""
        lib = load()
        n = C.c_int()
        check(lib.trvg_kernel_time_count(self._h, C.byref(n)))
        out = {}
        buf = C.create_string_buffer(64)
        for i in range(n.value):
            ms, cnt = C.c_double(), C.c_int64()
            check(lib.trvg_kernel_time_get(self._h, i, buf, 64, C.byref(ms),
                                           C.byref(cnt)))
            out[buf.value.decode()] = (ms.value, cnt.value)
        return out

    def tuned(self) -> dict:
        """{key: value} of the launch shapes the autotuner has chosen."""
        lib = load()
        n = C.c_int()
        check(lib.trvg_tuned_count(self._h, C.byref(n)))
        out = {}
        buf = C.create_string_buffer(128)
        for i in range(n.value):
            v = C.c_int64()
            check(lib.trvg_tuned_get(self._h, i, buf, 128, C.byref(v)))
            out[buf.value.decode()] = v.value
        return out

    def release_workspace(self):
        check(load().trvg_release_workspace(self._h))

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            load().trvg_context_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_ctx = {}


def default_context(device: int | None = None) -> Context:
    """Process-wide context of `device` (``TRVG_DEVICE``, default 0)."""
    if device is None:
        device = int(os.environ.get("TRVG_DEVICE", "0"))
    ctx = _default_ctx.get(device)
    if ctx is None:
        ctx = Context(device)
        _default_ctx[device] = ctx
    return ctx
