"""Array extrapolation used by the FFTLog transforms (mirror of the
reference's ``_arrayops.py``: ``extrap_pad``, ``extrap_lin``,
``extrap_loglin`` and their 2-d versions).

Each 1-d function returns the array with ``n_ext`` extra elements on either
side; the 2-d functions extend every row, then every column.
``extrap_loglin_oscil`` (extrapolation option 5) continues arrays that may
change sign or oscillate with a power law fitted to each tail.
"""
import warnings
from collections.abc import Sequence

import numpy as np


class DivergenceWarning(RuntimeWarning):
    """A tail grows outwards; it is padded with its end value instead."""


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


def _lngrad(a):
    """Gradient of log|a| (non-finite values set to 0, as nan_to_num)."""
    with np.errstate(divide='ignore', invalid='ignore'):
        return np.nan_to_num(np.gradient(np.log(np.abs(a))))


def _lngrad_raw(a):
    """Gradient of log|a| as it is (infinities and NaN kept)."""
    with np.errstate(divide='ignore', invalid='ignore'):
        return np.gradient(np.log(np.abs(a)))


def _changes(v):
    """Indices i where the sign of v changes between i and i + 1."""
    return np.nonzero(np.diff(np.sign(v)))[0]


def _oscil_tails(a):
    """Tail boundaries of the oscillatory extrapolation
    (_arrayops.py:332-409): the left tail is a[:lt], the right a[rt:];
    lq, rq bound the 'quarters' either side of the largest |a|."""
    n = a.size
    zero = _changes(a)  # sign changes of a
    lbank = max(zero[0] + 1, 3) if zero.size else n - 1
    rbank = min(zero[-1] + 1, n - 4) if zero.size else 0
    turn = _changes(_lngrad(a[:lbank]))  # extrema within the left bank
    ldbank = max(turn[-1] + 1, 3) if turn.size else n - 1
    turn = _changes(_lngrad(a[rbank:]))
    rdbank = min(rbank + turn[0], n - 4) if turn.size else 0
    peak = int(np.argmax(np.abs(a)))
    if peak in (0, n - 1):
        peak = n // 2
    lq = max((peak + 1) // 2 - 1, 3)
    rq = min(peak + (n - 1 - peak) // 2, n - 4)
    return min(lbank, ldbank, lq), max(rbank, rdbank, rq), lq, rq


def _tail_rate(trend, endpoint, fallback, side):
    """Power-law rate (per element, outwards) of one tail: the mean log
    gradient of an oscillating tail, else the end step, else the mean over
    the quarter; a tail that would grow outwards is padded (rate 0) with a
    DivergenceWarning.  `side` is +1 for the right tail, -1 for the left."""
    def outward(rate, what):
        if side * rate <= 0.:
            return side * rate
        warnings.warn(f"Divergent behaviour detected at the {what}. "
                      "Constant padding is used instead.",
                      DivergenceWarning, stacklevel=4)
        return 0.
    name = 'right' if side > 0 else 'left'
    if _changes(trend).size:
        return outward(float(np.mean(trend)), f"{name} tail")
    if side * endpoint <= 0.:
        return side * endpoint
    with np.errstate(invalid='ignore'):
        mean = float(np.nan_to_num(np.mean(fallback())))
    return outward(mean, f"{name} endpoints")


def extrap_loglin_oscil(a, n_ext):
    """Continue each tail of a possibly oscillating, sign-changing array
    with a power law exp(rate * i) from its end value
    (_arrayops.py:332-486): the rate is fitted on the tail outside the
    central peak and the innermost sign changes and turning points."""
    a = _as_1d(a)
    if a.size < 8:
        warnings.warn("Array length is less than 8. Extrapolation may not "
                      "be accurate.", UserWarning, stacklevel=2)
    lt, rt, lq, rq = _oscil_tails(a)
    with np.errstate(divide='ignore', invalid='ignore'):
        lend = float(np.nan_to_num(np.log(np.abs(a[1])) -
                                   np.log(np.abs(a[0]))))
        rend = float(np.nan_to_num(np.log(np.abs(a[-1])) -
                                   np.log(np.abs(a[-2]))))
    left = -_tail_rate(_lngrad(a[:lt]), lend, lambda: _lngrad_raw(a[:lq]),
                       -1)
    right = _tail_rate(_lngrad(a[rt:]), rend, lambda: _lngrad_raw(a[rq:]),
                       +1)
    # `left` is the outward (leftwards) decay rate per element.
    return np.concatenate([a[0] * np.exp(-left * np.arange(n_ext, 0, -1)),
                           a,
                           a[-1] * np.exp(right * np.arange(1, n_ext + 1))])


def _n2(n_ext):
    return tuple(n_ext) if isinstance(n_ext, Sequence) else (n_ext, n_ext)


def _rows_then_cols(a, n_ext, fn):
    a = _as_2d(a)
    nrow_ext, ncol_ext = _n2(n_ext)
    wide = np.array([fn(row, ncol_ext) for row in a])
    return np.array([fn(col, nrow_ext) for col in wide.T]).T


def extrap2d_loglin_oscil(a, n_ext):
    """Oscillatory log-linear continuation along rows, then columns."""
    return _rows_then_cols(a, n_ext, extrap_loglin_oscil)


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
