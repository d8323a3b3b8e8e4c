"""The correctly rounded log/exp/pow (and the turbulence closure's atan/cos) the CUDA kernels use (epic_gb300/csrc/dd_math.cuh),
host-compiled into the oracle's libepicport_cr.so, against 200-bit mpmath evaluations rounded
once to binary64, and their agreement with the host glibc (which the reference calls)."""
import ctypes as C
import math

import numpy as np
import pytest

from oracle_lib import PORT_CR_LIB, build_port

mpmath = pytest.importorskip("mpmath")


@pytest.fixture(scope="module")
def cr():
    build_port()
    lib = C.CDLL(PORT_CR_LIB)
    for n in ("epic_cr_log", "epic_cr_exp", "epic_cr_atan", "epic_cr_cos"):
        getattr(lib, n).restype = C.c_double
        getattr(lib, n).argtypes = [C.c_double]
    lib.epic_cr_pow.restype = C.c_double
    lib.epic_cr_pow.argtypes = [C.c_double, C.c_double]
    return lib


def _rn(v) -> float:
    """Round an mpmath value to the nearest binary64 (ties to even)."""
    return float(mpmath.mpf(v))   # mpf -> float rounds to nearest


def _inputs(seed, n):
    rng = np.random.default_rng(seed)
    x_log = np.concatenate([np.exp(rng.uniform(-30, 30, n)), 1. + rng.uniform(-1e-3, 1e-3, n // 4),
                            rng.uniform(10., 1.1e5, n // 2)])
    x_exp = np.concatenate([rng.uniform(-700, 700, n), rng.uniform(-1e-3, 1e-3, n // 4), rng.uniform(-12, 12, n // 2)])
    # the pow calls of the step: (p/p0)^kappa, p^(kappa+1), q^(1/kappa), cos(lat)^4
    kappa = 2. / 7.
    pw = [(x, kappa) for x in rng.uniform(1e-6, 1.1, n // 2)] + [(x, kappa + 1.) for x in rng.uniform(10., 1.1e5, n // 2)] + \
         [(x, 1. / kappa) for x in rng.uniform(1., 40., n // 2)] + [(x, 4.) for x in rng.uniform(0., 1., n // 4)] + \
         [(math.exp(a), b) for a, b in zip(rng.uniform(-12, 12, n), rng.uniform(-4, 4, n))]
    return x_log, x_exp, pw


def test_correctly_rounded_against_mpmath(cr):
    mpmath.mp.prec = 200
    x_log, x_exp, pw = _inputs(1, 4000)
    bad = [("log", x) for x in x_log if cr.epic_cr_log(float(x)) != _rn(mpmath.log(mpmath.mpf(float(x))))]
    bad += [("exp", x) for x in x_exp if cr.epic_cr_exp(float(x)) != _rn(mpmath.exp(mpmath.mpf(float(x))))]
    bad += [("pow", x, y) for x, y in pw if x > 0 and
            cr.epic_cr_pow(float(x), float(y)) != _rn(mpmath.power(mpmath.mpf(float(x)), mpmath.mpf(float(y))))]
    assert not bad, bad[:5]


def test_agreement_with_host_libm(cr):
    """glibc's log/exp/pow are correctly rounded in all but a small fraction of calls; the
    differences are those calls (so the kernels and the reference differ in those cells)."""
    x_log, x_exp, pw = _inputs(2, 20000)
    d_log = np.mean([cr.epic_cr_log(float(x)) != math.log(x) for x in x_log])
    d_exp = np.mean([cr.epic_cr_exp(float(x)) != math.exp(x) for x in x_exp])
    d_pow = np.mean([cr.epic_cr_pow(float(x), float(y)) != math.pow(x, y) for x, y in pw])
    assert d_log < 5e-3 and d_exp < 5e-3 and d_pow < 5e-3, (d_log, d_exp, d_pow)


def test_turbulence_functions_correctly_rounded(cr):
    """atan (the wall law's, arguments sqrt(1/3) (2 yy - 1) with yy in [0.635, 8.9), and any sign
    and size), cos (invert_fv1's, |x| < 0.2, and |x| < 1) and the powers the closure takes
    (x^2 of any sign -- the square rounded once --, x^3, x^6, x^(1/6), x^0.35, x^0.25, x^4)."""
    mpmath.mp.prec = 200
    rng = np.random.default_rng(5)
    xa = np.concatenate([rng.uniform(0.15, 9.7, 2000), rng.uniform(-50, 50, 1000), np.exp(rng.uniform(-40, 40, 1000))])
    xc = np.concatenate([rng.uniform(0.03, 0.2, 2000), rng.uniform(-0.999, 0.999, 1000)])
    bad = [("atan", x) for x in xa if cr.epic_cr_atan(float(x)) != _rn(mpmath.atan(mpmath.mpf(float(x))))]
    bad += [("cos", x) for x in xc if cr.epic_cr_cos(float(x)) != _rn(mpmath.cos(mpmath.mpf(float(x))))]
    pw = [(x, 2.) for x in rng.uniform(-1e3, 1e3, 1000)] + [(x, 3.) for x in rng.uniform(1e-3, 1e3, 500)] + \
         [(x, 6.) for x in rng.uniform(1e-2, 10., 500)] + [(x, 1. / 6.) for x in rng.uniform(0.1, 2., 500)] + \
         [(x, 0.35) for x in rng.uniform(0.4, 30., 500)] + [(x, .25) for x in rng.uniform(1e-3, 160., 500)] + \
         [(x, 4.) for x in rng.uniform(5., 70., 500)]
    bad += [("pow", x, y) for x, y in pw
            if cr.epic_cr_pow(float(x), float(y)) != _rn(mpmath.power(mpmath.mpf(float(x)), mpmath.mpf(float(y))))]
    assert not bad, bad[:5]
