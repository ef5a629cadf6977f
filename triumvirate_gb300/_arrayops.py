"""Array extrapolation used by the FFTLog transforms (mirror of the
reference's ``_arrayops.py``: ``extrap_pad``, ``extrap_lin``,
``extrap_loglin`` and their 2-d versions).

Each 1-d function returns the array with ``n_ext`` extra elements on either
side; the 2-d functions extend every row, then every column.  The
oscillatory log-linear scheme (``extrap_loglin_oscil``, extrapolation
option 5 of the transforms) is not provided.
"""
from collections.abc import Sequence

import numpy as np


def _as_nd(a, ndim):
    """Float array (complex kept) of `ndim` dimensions."""
    a = np.asarray(a)
    a = a.astype(complex if np.iscomplexobj(a) else float)
    if a.ndim != ndim:
        raise ValueError(f"Input array must be {ndim}-d.")
    return a


def _as_1d(a):
    return _as_nd(a, 1)


def _as_2d(a):
    return _as_nd(a, 2)


def extrap_pad(a, n_ext, c_lower, c_upper):
    """Pad with the constants `c_lower` (left) and `c_upper` (right)."""
    a = _as_1d(a)
    return np.concatenate([np.full(n_ext, c_lower, dtype=a.dtype), a,
                           np.full(n_ext, c_upper, dtype=a.dtype)])


def extrap_lin(a, n_ext):
    """Continue the first and last steps linearly."""
    a = _as_1d(a)
    left = a[0] + np.arange(-n_ext, 0) * (a[1] - a[0])
    right = a[-1] + np.arange(1, n_ext + 1) * (a[-1] - a[-2])
    return np.concatenate([left, a, right])


def extrap_loglin(a, n_ext):
    """Continue the first and last log steps (values of one sign, no
    zeros)."""
    a = _as_1d(a)
    if np.iscomplexobj(a):
        if np.any(a == 0.):
            raise ValueError("Zeros detected in the input array.")
    elif np.any(a[:-1] * a[1:] <= 0.):
        raise ValueError("Sign change or zeros detected in the input array.")
    left = a[0] * np.exp(np.arange(-n_ext, 0) * np.log(a[1] / a[0]))
    right = a[-1] * np.exp(np.arange(1, n_ext + 1) * np.log(a[-1] / a[-2]))
    return np.concatenate([left, a, right])


def extrap_loglin_oscil(a, n_ext):
    """Not provided: the transforms accept extrapolation options 0-4."""
    raise NotImplementedError(
        "Oscillatory log-linear extrapolation (option 5) is not provided.")


def _n2(n_ext):
    return tuple(n_ext) if isinstance(n_ext, Sequence) else (n_ext, n_ext)


def _rows_then_cols(a, n_ext, fn):
    a = _as_2d(a)
    nrow_ext, ncol_ext = _n2(n_ext)
    wide = np.array([fn(row, ncol_ext) for row in a])
    return np.array([fn(col, nrow_ext) for col in wide.T]).T


def extrap2d_lin(a, n_ext):
    """Linear continuation along rows, then along columns."""
    return _rows_then_cols(a, n_ext, extrap_lin)


def extrap2d_loglin(a, n_ext):
    """Log-linear continuation along rows, then along columns."""
    return _rows_then_cols(a, n_ext, extrap_loglin)


def extrap2d_pad(a, n_ext, crow_lower, crow_upper, ccol_lower, ccol_upper):
    """Constant padding: rows get `crow_lower` / `crow_upper` at their ends
    (scalars or one per row), then the column ends `ccol_lower` /
    `ccol_upper` (scalars or one per original column; the corner values
    continue the row paddings)."""
    a = _as_2d(a)
    nrow_ext, ncol_ext = _n2(n_ext)
    nr, nc = a.shape
    rl = np.broadcast_to(np.asarray(crow_lower, float), (nr,))
    ru = np.broadcast_to(np.asarray(crow_upper, float), (nr,))
    cl = np.broadcast_to(np.asarray(ccol_lower, float), (nc,))
    cu = np.broadcast_to(np.asarray(ccol_upper, float), (nc,))
    if rl[0] != cl[0] or ru[0] != cl[-1] or rl[-1] != cu[0] \
            or ru[-1] != cu[-1]:
        raise ValueError("Inconsistent padding values for rows and columns.")
    wide = np.hstack([np.repeat(rl[:, None], ncol_ext, 1), a,
                      np.repeat(ru[:, None], ncol_ext, 1)])
    top = np.concatenate([np.full(ncol_ext, rl[0]), cl, np.full(ncol_ext,
                                                               ru[0])])
    bot = np.concatenate([np.full(ncol_ext, rl[-1]), cu,
                          np.full(ncol_ext, ru[-1])])
    return np.vstack([np.repeat(top[None, :], nrow_ext, 0), wide,
                      np.repeat(bot[None, :], nrow_ext, 0)])
