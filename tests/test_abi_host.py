"""The C-ABI library without a GPU: it loads, exports every symbol declared
in ``include/trvg.h``, and its host maths (the same code the kernels run)
matches the oracle."""
import re
from pathlib import Path

import numpy as np
import pytest
from scipy.special import spherical_jn

from oracle import trv_oracle as O
from triumvirate_gb300 import _lib

HEADER = Path(__file__).resolve().parents[1] / "include" / "trvg.h"


def _declared():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"\b(trvg_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    names = _declared()
    assert len(names) >= 19
    for name in names:
        assert hasattr(lib, name), name
    assert sorted(_lib.EXPORTED) == names


def test_version():
    assert b"sm_103a" in _lib.load().trvg_version()


@pytest.mark.parametrize("args", [
    (0, 0, 0, 0, 0, 0), (2, 0, 2, 0, 0, 0), (2, 0, 2, 1, 0, -1),
    (2, 0, 2, -2, 0, 2), (1, 1, 2, 1, -1, 0), (2, 2, 2, 0, 0, 0),
    (3, 2, 1, -2, 1, 1), (4, 4, 4, 2, -1, -1), (2, 2, 1, 0, 0, 0),
    (6, 4, 2, 3, -2, -1), (1, 1, 1, 1, 1, 1)])
def test_wigner_3j(args):
    assert abs(_lib.load().trvg_wigner_3j(*args) - O.wigner_3j(*args)) \
        < 1e-14


@pytest.mark.parametrize("ell", [0, 1, 2, 3, 4, 6, 8])
def test_sph_bessel_against_scipy(ell):
    lib = _lib.load()
    xs = np.concatenate([np.linspace(0., 5., 501)[1:],
                         np.linspace(5., 1000., 997), [1e-6, 1e-3, 0.05]])
    got = np.array([lib.trvg_sph_bessel(ell, float(x)) for x in xs])
    ref = spherical_jn(ell, xs)
    assert np.max(np.abs(got - ref)) < 2e-15


@pytest.mark.parametrize("ell", [0, 1, 2, 4])
def test_bessel_spline_matches_oracle_spline(ell):
    """The kernels' natural cubic spline (maths.cpp:309-375) equals the
    oracle's natural spline through the same nodes."""
    rng = np.random.default_rng(ell)
    xs = np.concatenate([rng.uniform(0., 1000., 4000),
                         0.05 * np.arange(0, 20001, 997),
                         [999.99, 1000., 1000.5, 1500.]])
    out = np.zeros_like(xs)
    _lib.check(_lib.load().trvg_sph_bessel_spline(
        ell, _lib.dptr(xs), xs.size, _lib.dptr(out)))
    ref = O.SphericalBessel(ell).eval(xs)
    assert np.max(np.abs(out - ref)) < 1e-13


@pytest.mark.parametrize("ell, m", [(0, 0), (1, -1), (1, 0), (1, 1),
                                    (2, -2), (2, -1), (2, 0), (2, 1),
                                    (2, 2), (3, -3), (4, 3)])
def test_reduced_ylm_matches_oracle(ell, m):
    rng = np.random.default_rng(100 + 10 * ell + m)
    v = rng.normal(size=(500, 3))
    v[0] = [0., 0., 0.]          # |v| < 1e-9 -> 0
    v[1] = [0., 0., 2.]          # on the z axis: phi = 0
    v[2] = [1e-12, 0., -1.]
    v[3] = [0.3, -0.4, 0.]       # y < 0 branch
    v = np.ascontiguousarray(v)
    out = np.zeros(2 * v.shape[0])
    _lib.check(_lib.load().trvg_reduced_ylm(ell, m, _lib.dptr(v), v.shape[0],
                                            _lib.dptr(out)))
    got = out[0::2] + 1j * out[1::2]
    ref = O.reduced_ylm(ell, m, v)
    # The oracle follows the reference's phi = arccos(x / r_xy), which loses
    # digits near phi = 0, pi; the kernels form exp(i m phi) from
    # (x + i y) / r_xy.  Agreement is to ~1e-13 away from those points.
    assert np.max(np.abs(got - ref)) < 1e-11


def test_data_vector_dim():
    import ctypes as C
    lib = _lib.load()
    d = C.c_int()
    for shape, nb, idx, exp in [(0, 20, 0, 20), (1, 20, 3, 17), (1, 20, -3, 17),
                                (2, 20, 4, 20), (3, 20, 0, 400),
                                (4, 20, 0, 210)]:
        _lib.check(lib.trvg_data_vector_dim(shape, nb, idx, C.byref(d)))
        assert d.value == exp
    with pytest.raises(_lib.InvalidParameterError):
        _lib.check(lib.trvg_data_vector_dim(9, 20, 0, C.byref(d)))


def test_invalid_spline_argument_is_an_error():
    xs = np.array([-1.])
    out = np.zeros(1)
    with pytest.raises(_lib.InvalidParameterError):
        _lib.check(_lib.load().trvg_sph_bessel_spline(
            0, _lib.dptr(xs), 1, _lib.dptr(out)))
