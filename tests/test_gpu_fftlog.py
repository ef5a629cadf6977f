"""GPU FFTLog (trvg_hankel_*) against the oracle and the analytic pairs of
the reference's tests/test_transforms.py."""
import numpy as np
import pytest

from oracle import trv_oracle as O
from test_fftlog import (HANKEL_CASES, HANKEL_PAIRS, SJ_CASES, SJ_PAIRS,
                         oracle_sbt)
from triumvirate_gb300 import _lib
from triumvirate_gb300._fftlog import HankelTransform
from triumvirate_gb300.transforms import (DoubleSphericalBesselTransform,
                                          SphericalBesselTransform)

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("order, bias, n, lg, extrap, pair, lgt", HANKEL_CASES)
def test_hankel_matches_oracle_and_analytic(order, bias, n, lg, extrap, pair,
                                            lgt):
    f, g = HANKEL_PAIRS[pair]
    x = np.logspace(*lg, n, base=10, endpoint=False)
    ht = HankelTransform(order, bias, x, kr_c=1., lowring=True, extrap=extrap)
    k, b = ht.transform(f(x, order))
    ko, bo = O.hankel_transform(order, bias, x, f(x, order), extrap=extrap)
    assert np.allclose(k, ko, rtol=1e-13, atol=0)
    assert ht.pivot == pytest.approx(
        O.fftlog_lowring_pivot(order, bias, ht._logres, 1.), rel=1e-12)
    assert np.max(np.abs(b - bo)) <= 1e-10 * np.max(np.abs(bo))
    sel = (lgt[0] < np.log10(k)) & (np.log10(k) < lgt[-1])
    assert np.allclose(b[sel].real, g(k, order)[sel], rtol=1e-3)


def test_hankel_batch_rows_equal_single_rows():
    x = np.logspace(-4., 4., 512, base=10, endpoint=False)
    rows = np.array([x ** (1.5 + 0.1 * i) * np.exp(-x * x / (2. + i))
                     for i in range(6)])
    ht = HankelTransform(1.5, 0.3, x, kr_c=0., lowring=True)
    _, batch = ht.transform(rows)
    for i, r in enumerate(rows):
        _, one = ht.transform(r)
        assert np.array_equal(batch[i], one)
        _, ref = O.hankel_transform(1.5, 0.3, x, r, kr_c=0.)
        assert np.max(np.abs(one - ref)) <= 1e-10 * np.max(np.abs(ref))


@pytest.mark.parametrize("ell, bias, n, lg, extrap, pair, lgt", SJ_CASES)
def test_sbt_matches_oracle_and_analytic(ell, bias, n, lg, extrap, pair, lgt):
    f, g = SJ_PAIRS[pair]
    x = np.logspace(*lg, n, base=10, endpoint=False)
    sbt = SphericalBesselTransform(ell, bias, x, lowring=True, extrap=extrap)
    k, b = sbt.transform(f(x, ell))
    ko, bo = oracle_sbt(ell, bias, x, f(x, ell), extrap)
    assert np.allclose(k, ko, rtol=1e-13, atol=0)
    # Compared before the post-factor (2 pi / k)^{3/2}, which reaches 1e8 at
    # the smallest k and magnifies the FP64 FFT rounding of either side.
    h, ho = b * (k / (2 * np.pi)) ** 1.5, bo * (k / (2 * np.pi)) ** 1.5
    assert np.max(np.abs(h - ho)) <= 1e-10 * np.max(np.abs(ho))
    sel = (lgt[0] < np.log10(k)) & (np.log10(k) < lgt[-1])
    assert np.allclose(b[sel].real, g(k, ell)[sel], rtol=1e-3)
    # Forward cosmological multipole: i^-l times the transform.
    _, c = sbt.transform_cosmo_multipoles('forward', f(x, ell))
    assert np.allclose(c, (-1j) ** ell * b, rtol=1e-12, atol=0)


@pytest.mark.parametrize("degrees, n, extrap, pair, lgt", [
    ((0, 0), 2 ** 10, 0, 'sym', (-3., 0.)),
    ((2, 2), 2 ** 11, 4, 'asym', (-.5, 3.)),
])
def test_double_sbt_analytic(degrees, n, extrap, pair, lgt):
    """Reference tests/test_transforms.py:101-141."""
    f, g = SJ_PAIRS[pair]
    x = np.logspace(-5., 5., n, base=10, endpoint=False)
    pre = f(x, degrees[0])[:, None] * f(x, degrees[1])[None, :]
    t = DoubleSphericalBesselTransform(degrees, (0, 0), x, lowring=True,
                                       extrap=extrap)
    (k0, k1), post = t.transform(pre)
    expect = g(k0, degrees[0]) * g(k1, degrees[1])
    sel = np.logical_and.reduce([np.log10(k0) > lgt[0],
                                 np.log10(k0) < lgt[-1],
                                 np.log10(k1) > lgt[0],
                                 np.log10(k1) < lgt[-1]])
    assert np.allclose(post[sel].real, expect[sel], rtol=1e-3)


def test_hankel_invalid_inputs_raise():
    x = np.logspace(-2., 2., 64)
    with pytest.raises(_lib.InvalidParameterError):
        HankelTransform(0., 0., x[:-1], kr_c=1., extrap=4)  # odd size
    with pytest.raises(_lib.InvalidParameterError):
        HankelTransform(0., 0., np.linspace(1., 2., 64), kr_c=1.)
    with pytest.raises(_lib.InvalidParameterError):
        HankelTransform(-1., 0., x, kr_c=1.)  # pole of the gamma function
