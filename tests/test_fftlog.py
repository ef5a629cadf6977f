"""FFTLog oracle and array helpers on the CPU, against the analytic
transform pairs of the reference's tests (tests/test_transforms.py:14-141,
rtol 1e-3 in the stated ranges) and its resampling tests."""
import numpy as np
import pytest
from scipy.special import gamma

from oracle import trv_oracle as O
from triumvirate_gb300 import _arrayops as A
from triumvirate_gb300.transforms import resample_lglin, resample_lin

HANKEL_PAIRS = {
    'sym': (lambda r, mu: r ** (mu + 1.) * np.exp(-r * r / 2.),
            lambda k, mu: k ** (mu + 1.) * np.exp(-k * k / 2.)),
    'asym': (lambda r, mu: r * (1. + r ** 2) ** (-1.5),
             lambda k, mu: k * np.exp(-k)),
}
SJ_PAIRS = {
    'sym': (lambda r, ell: r ** ell * np.exp(-r * r / 2.),
            lambda k, ell: k ** ell * np.exp(-k * k / 2.)
            * (2 * np.pi) ** 1.5),
    'asym': (lambda r, ell, s=1: r ** (s - 3),
             lambda k, ell, s=1: np.pi ** 1.5 * gamma(s / 2. + ell / 2.)
             / gamma(1.5 - s / 2. + ell / 2.) * (2. / k) ** s),
}
HANKEL_CASES = [(2, 0, 2 ** 10, (-5., 5.), 0, 'sym', (-3., .5)),
                (0, 0, 2 ** 11, (-5., 5.), 4, 'asym', (-3., .5))]
SJ_CASES = [(0, 0, 2 ** 10, (-5., 5.), 0, 'sym', (-3.5, .5)),
            (2, 0, 2 ** 11, (-5., 5.), 4, 'asym', (-1., 3.))]


def oracle_sbt(ell, q, x, f, extrap):
    """Spherical-Bessel transform from the oracle's Hankel transform with
    the reference's 'outer' extension and r^{3/2}, (2 pi / k)^{3/2}."""
    n_ext = 0
    if extrap:
        n_ext = (int(2 ** np.ceil(np.log2(2. * len(x)))) - len(x)) // 2
        x = A.extrap_loglin(x, n_ext)
        f = A.extrap_loglin(f, n_ext)
    k, g = O.hankel_transform(ell + 0.5, q, x, f * x ** 1.5)
    sl = slice(n_ext, -n_ext) if n_ext else slice(None)
    return k[sl], g[sl] * (2 * np.pi / k[sl]) ** 1.5


@pytest.mark.parametrize("order, bias, n, lg, extrap, pair, lgt", HANKEL_CASES)
def test_oracle_hankel_analytic(order, bias, n, lg, extrap, pair, lgt):
    f, g = HANKEL_PAIRS[pair]
    x = np.logspace(*lg, n, base=10, endpoint=False)
    k, b = O.hankel_transform(order, bias, x, f(x, order), extrap=extrap)
    sel = (lgt[0] < np.log10(k)) & (np.log10(k) < lgt[-1])
    assert np.allclose(b[sel].real, g(k, order)[sel], rtol=1e-3)


@pytest.mark.parametrize("ell, bias, n, lg, extrap, pair, lgt", SJ_CASES)
def test_oracle_sbt_analytic(ell, bias, n, lg, extrap, pair, lgt):
    f, g = SJ_PAIRS[pair]
    x = np.logspace(*lg, n, base=10, endpoint=False)
    k, b = oracle_sbt(ell, bias, x, f(x, ell), extrap)
    sel = (lgt[0] < np.log10(k)) & (np.log10(k) < lgt[-1])
    assert np.allclose(b[sel].real, g(k, ell)[sel], rtol=1e-3)


def test_extrapolation_helpers():
    a = np.array([1., 2., 4., 8.])
    assert np.array_equal(A.extrap_pad(a, 2, 0., 9.),
                          [0, 0, 1, 2, 4, 8, 9, 9])
    assert np.allclose(A.extrap_lin(a, 2), [-1, 0, 1, 2, 4, 8, 12, 16])
    assert np.allclose(A.extrap_loglin(a, 2), [.25, .5, 1, 2, 4, 8, 16, 32])
    with pytest.raises(ValueError):
        A.extrap_loglin(np.array([1., -1., 2.]), 1)
    with pytest.warns(UserWarning, match="less than 8"):
        assert A.extrap_loglin_oscil(np.arange(1., 9.)[:6], 1).shape == (8,)
    m = np.outer([1., 2.], [1., 3.])
    e = A.extrap2d_loglin(m, 1)
    assert e.shape == (4, 4)
    assert np.allclose(e, np.outer([.5, 1., 2., 4.], [1. / 3, 1., 3., 9.]))
    assert np.allclose(A.extrap2d_lin(m, (1, 1))[1:-1, 1:-1], m)
    p = A.extrap2d_pad(m, 1, 0., 0., 0., 0.)
    assert p.shape == (4, 4) and p[0].sum() == 0 and p[:, 0].sum() == 0


@pytest.mark.parametrize("sampts, size, func, ndim", [
    (np.arange(1., 11.), None, lambda x: x ** 2, 1),
    (np.arange(1., 51.) * 1.e-3, 10, lambda x, y: np.exp(-x * np.sqrt(y)), 2),
])
def test_resampling(sampts, size, func, ndim):
    """Reference tests/test_transforms.py:143-200."""
    for fn in (resample_lglin, resample_lin):
        if ndim == 1:
            rs, rv = fn(sampts, func(sampts), size=size)
            assert np.allclose(rv, func(rs))
        else:
            samples = func(*np.meshgrid(sampts, sampts, indexing='ij'))
            rs, rv = fn(sampts, samples, size=size)
            assert np.allclose(rv, func(*np.meshgrid(rs[0], rs[-1],
                                                     indexing='ij')))


def test_extrap_loglin_oscil_matches_reference_goldens():
    """Extrapolation option 5 against the reference's own outputs on its
    branches: oscillating and monotonic tails, tails growing outwards
    (constant padding with a DivergenceWarning), sign changes and zeros
    (tests/golden/make_extrap_fixtures.py)."""
    import warnings
    from pathlib import Path

    from triumvirate_gb300._arrayops import (DivergenceWarning,
                                             extrap2d_loglin_oscil,
                                             extrap_loglin_oscil)
    d = np.load(Path(__file__).resolve().parent / "golden" /
                "extrap_loglin_oscil.npz")
    names = sorted({k.split("__")[0] for k in d.files})
    assert len(names) == 8
    for name in names:
        with warnings.catch_warnings(record=True) as caught:
            warnings.simplefilter("always")
            got = extrap_loglin_oscil(d[name + "__in"], 16)
        assert np.array_equal(got, d[name + "__out"]), name
        if name == "growing_tails":
            assert any(issubclass(w.category, DivergenceWarning)
                       for w in caught)
    # 2-d: rows, then columns.
    a = np.outer(d["damped_oscillation__in"][:12], d["power_law__in"][:10])
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        out = extrap2d_loglin_oscil(a, (3, 4))
        rows = np.array([extrap_loglin_oscil(r, 4) for r in a])
        ref = np.array([extrap_loglin_oscil(c, 3) for c in rows.T]).T
    assert out.shape == (18, 18) and np.array_equal(out, ref)
