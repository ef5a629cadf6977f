"""FFTLog Hankel transform (mirror of the reference's ``_fftlog.pyx``,
``trv::maths::HankelTransform``, include/fftlog.hpp:68-257).

The plan (pivot, kernel coefficients, sample points) is built by the C ABI
(``trvg_hankel_create``); transforms run on the GPU, and a 2-d input is
transformed row by row in one batched call.
"""
import ctypes as C

import numpy as np

from . import _lib


class HankelTransform:
    """Forward biased Hankel transform
    ``b(k) = int_0^inf k dr (k r)^q J_mu(k r) a(r)`` by FFTLog.

    Parameters as in the reference: order `mu`, bias `q`, log-spaced
    sample points `x`, pivot `kr_c`, `lowring`, native extrapolation option
    `extrap` (0-4) and size factor `extrap_exp`; `threaded` is accepted for
    compatibility.
    """

    def __init__(self, mu, q, x, kr_c, lowring=True, extrap=0,
                 extrap_exp=2., threaded=False, device=None):
        x = np.ascontiguousarray(x, dtype=np.float64).copy()
        lib = _lib.load()
        h = C.c_void_p()
        _lib.check(lib.trvg_hankel_create(
            float(mu), float(q), _lib.dptr(x), int(x.size), float(kr_c),
            int(bool(lowring)), int(extrap or 0), float(extrap_exp),
            C.byref(h)))
        self._h = h
        self._ctx = _lib.default_context(device)
        n, nt = C.c_int(), C.c_int()
        piv, lr = C.c_double(), C.c_double()
        pre = np.empty(x.size)
        post = np.empty(x.size)
        _lib.check(lib.trvg_hankel_info(
            h, C.byref(n), C.byref(nt), C.byref(piv), C.byref(lr),
            _lib.dptr(pre), _lib.dptr(post)))
        self.order = float(mu)
        self.bias = float(q)
        self._nsamp = n.value
        self._nsamp_trans = nt.value
        self._logres = lr.value
        self._pivot = piv.value
        self._pre_sampts = pre
        self._post_sampts = post

    def __del__(self):
        h = getattr(self, '_h', None)
        if h is not None and h.value is not None:
            _lib.load().trvg_hankel_destroy(h)
            self._h = None

    @property
    def size(self):
        """Sample size of the transform."""
        return self._nsamp_trans

    @property
    def pivot(self):
        """Pivot value used."""
        return self._pivot

    def transform(self, fx):
        """Transform samples at the initialised points: `fx` of shape (n,)
        or (rows, n); returns the post-transform points and samples."""
        fx = np.asarray(fx)
        rows = fx.reshape(-1, self._nsamp).astype(np.complex128)
        a = np.ascontiguousarray(rows).view(np.float64)
        b = np.empty_like(a)
        _lib.check(_lib.load().trvg_hankel_transform(
            self._ctx.handle, self._h, int(rows.shape[0]), _lib.dptr(a),
            _lib.dptr(b)))
        gy = b.view(np.complex128).reshape(fx.shape)
        return np.array(self._post_sampts), gy
