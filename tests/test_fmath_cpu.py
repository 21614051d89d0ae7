"""Accuracy of the portable FP64 exp / log / log10 / pow / sin / cos
(mcx_fmath.h) that the device's FP64 balance and transport and the oracle's
share: within a few ulp of the
host's libm (numpy) over the ranges the balance evaluates, plus the C99
special cases.  pow = exp(y ln x) carries the relative error of y ln x into
its result, about 2 |y ln x| ulp (1e-14 for Te^-1.5 at 1e4 K)."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.filterwarnings("ignore::RuntimeWarning")


def _ulps(a, b):
    """|a - b| in units of the last place of b."""
    return np.abs(a - b) / np.spacing(np.abs(b))


@pytest.fixture(scope="module")
def rng():
    oracle.build()
    return np.random.default_rng(20261204)


def test_exp(rng):
    x = np.concatenate([rng.uniform(-745, 709.7, 200000), rng.uniform(-1, 1, 100000), rng.uniform(-50, 50, 100000),
                        [0.0, -0.0, 1.0, -1.0, 1e-300, -1e-300, 700.0, -700.0, -740.0]])
    got = oracle.fm_eval(oracle.FM_EXP, x)
    ref = np.exp(x)
    normal = ref > 2.3e-308
    assert _ulps(got[normal], ref[normal]).max() <= 2.0
    # subnormal results: one rounding into the subnormal range
    sub = (ref > 0) & ~normal
    assert np.all(np.abs(got[sub] - ref[sub]) <= 2 * 4.95e-324)
    assert oracle.fm_eval(oracle.FM_EXP, np.array([710.0]))[0] == np.inf
    assert oracle.fm_eval(oracle.FM_EXP, np.array([-746.0]))[0] == 0.0
    assert np.isnan(oracle.fm_eval(oracle.FM_EXP, np.array([np.nan]))[0])


def test_log_log10(rng):
    x = np.concatenate([10.0 ** rng.uniform(-307, 308, 200000), rng.uniform(0.5, 2.0, 100000),
                        1.0 + rng.uniform(-1e-6, 1e-6, 10000), [1.0, 2.0, 0.5, 10.0, 1e4, 5e-324, 1e-310]])
    got = oracle.fm_eval(oracle.FM_LOG, x)
    ref = np.log(x)
    nz = ref != 0
    assert _ulps(got[nz], ref[nz]).max() <= 2.0
    assert oracle.fm_eval(oracle.FM_LOG, np.array([1.0]))[0] == 0.0
    g10 = oracle.fm_eval(oracle.FM_LOG10, x)
    r10 = np.log10(x)
    nz = r10 != 0
    assert _ulps(g10[nz], r10[nz]).max() <= 3.0
    sp = oracle.fm_eval(oracle.FM_LOG, np.array([0.0, -1.0, np.inf, np.nan]))
    assert sp[0] == -np.inf and np.isnan(sp[1]) and sp[2] == np.inf and np.isnan(sp[3])


def test_pow(rng):
    # the balance's uses: Te^(+-1.5), Te/T0 ^ (fit exponents), (1 - x^a)^b, 10^(poly in log10 Te)
    x = np.concatenate([10.0 ** rng.uniform(-6, 9, 100000), rng.uniform(0, 1, 50000), [10.0] * 1000])
    y = np.concatenate([rng.uniform(-3, 3, 100000), rng.uniform(0.1, 2, 50000), rng.uniform(-30, 20, 1000)])
    got = oracle.fm_eval(oracle.FM_POW, x, y)
    ref = np.power(x, y)
    ok = (ref > 1e-300) & (ref < 1e300)
    bound = 2.0 * np.abs(y * np.log(x)) + 4.0
    assert np.all(_ulps(got[ok], ref[ok]) <= bound[ok])
    sx = np.array([0.0, 0.0, -2.0, -2.0, -2.0, 1.0, np.nan, 2.0, 0.5, 5.0, -0.0])
    sy = np.array([2.0, -1.0, 3.0, 2.0, 0.5, np.nan, 0.0, np.inf, np.inf, -np.inf, 3.0])
    g = oracle.fm_eval(oracle.FM_POW, sx, sy)
    assert g[0] == 0.0 and g[1] == np.inf and np.isnan(g[4])
    assert g[2] == pytest.approx(-8.0, rel=1e-14) and g[3] == pytest.approx(4.0, rel=1e-14)
    assert g[5] == 1.0 and g[6] == 1.0 and g[7] == np.inf and g[8] == 0.0 and g[9] == 0.0 and g[10] == 0.0
    # integral exponents of the balance (x**2, x**3 of the fits)
    xi = 10.0 ** rng.uniform(-5, 5, 10000)
    for k in (2.0, 3.0, -1.0, 0.5):
        assert np.all(_ulps(oracle.fm_eval(oracle.FM_POW, xi, np.full_like(xi, k)), xi ** k)
                      <= 2.0 * np.abs(k * np.log(xi)) + 4.0)


def test_sin_cos(rng):
    x = np.concatenate([rng.uniform(-np.pi, np.pi, 200000), rng.uniform(-1e3, 1e3, 50000),
                        rng.uniform(-1e-3, 1e-3, 10000), [0.0, np.pi / 2, -np.pi, np.pi, 3.141592654]])
    for fn, ref in ((oracle.FM_SIN, np.sin), (oracle.FM_COS, np.cos)):
        got = oracle.fm_eval(fn, x)
        want = ref(x)
        # near a zero of the function the absolute error of the pi/2 reduction
        # (about k 1e-26) sets the bound
        assert np.all(np.abs(got - want) <= 2.0 * np.spacing(np.abs(want)) + 1e-22), fn
    assert np.isnan(oracle.fm_eval(oracle.FM_SIN, np.array([np.inf]))[0])
