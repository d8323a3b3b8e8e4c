"""The mixed-precision form (EPIC_PREC_MIXED) against the FP64 form on the GPU.

Mixed form: stencils, advection, hyperviscosity, the pressure gradient, the zonal filter (on the
tensor cores for ni a multiple of 128) and the physics evaluate in FP32; the hydrostatic sums
(P3, GZ3, SUM_DIV), the row means, every update of a stored field and the Adams-Bashforth/
leapfrog step stay FP64 (the state is stored in FP64).

Stated error (relative L2 per field, mixed vs FP64), measured on a GB300:
  * one simulated day (288 steps of 300 s) at 64x32x10 from a state spun up for 10 days:
    U 3.5e-5, V 3.9e-4, HDRY 2.6e-7, THETA 3.7e-8;
  * one simulated day from rest: U 2.2e-4, V 5.9e-4 (the first days are driven by horizontal
    pressure differences 1e-5 of the geopotential, so FP32 rounding is amplified ~1e4 in U, V).
The bounds below leave a factor ~3 over those figures.
"""
import numpy as np
import pytest

from compare import PROGNOSTIC, field_errors
from epic_gb300 import EPIC_PREC_FP64, EPIC_PREC_MIXED, EPIC_SYNC_DIAGS_ONLY, EPIC_UV_LEAPFROG, HSConfig, Model, hs_setup

pytestmark = pytest.mark.gpu
DAY = 288   # steps of 300 s


@pytest.fixture(scope="module")
def spun_up(gpu):
    ga, f = hs_setup(HSConfig(ni=64, nj=32, nk=10, dt=300, seed=0))
    m = Model(ga, EPIC_PREC_FP64)
    m.upload(f)
    m.timestep(EPIC_SYNC_DIAGS_ONLY)
    m.run(10 * DAY)
    m.sync()
    return ga, m.download()


def _pair(ga, f, prime):
    a, b = Model(ga, EPIC_PREC_FP64), Model(ga, EPIC_PREC_MIXED)
    for m in (a, b):
        m.upload(f)
        if prime:
            m.timestep(EPIC_SYNC_DIAGS_ONLY)
    return a, b


def _run(a, b, n):
    a.run(n)
    b.run(n)
    a.sync()
    b.sync()
    return field_errors(b.download(), a.download(), PROGNOSTIC)


def test_mixed_one_day_after_spin_up(spun_up):
    ga, f = spun_up
    a, b = _pair(ga, f, prime=False)
    e = _run(a, b, DAY)
    bounds = {"u": 1e-4, "v": 1e-3, "hdry": 1e-6, "theta": 1e-7}
    assert all(e[k][0] <= bounds[k] for k in bounds), e


def test_mixed_one_day_from_rest(gpu):
    ga, f = hs_setup(HSConfig(ni=64, nj=32, nk=10, dt=300, seed=0))
    a, b = _pair(ga, f, prime=True)
    e = _run(a, b, DAY)
    bounds = {"u": 1e-3, "v": 2e-3, "hdry": 1e-6, "theta": 1e-7}
    assert all(e[k][0] <= bounds[k] for k in bounds), e


def test_mixed_leapfrog_follows_fp64(gpu):
    """The leapfrog (Asselin-filtered) wind step in the mixed form, 12 simulated hours from rest
    (measured on a GB300: U 1.6e-3, V 5.0e-4, HDRY 1.5e-7, THETA 3.7e-8; the U, V errors are
    those of the AB3 form at the same time, where the winds are still weak).  The FP64 leapfrog
    run of this configuration itself stops with non-monotonic GZ3 between the first and second
    day, so the comparison ends before.  The time-plane bookkeeping (IT_ZERO, itime) must be the
    FP64 form's."""
    ga, f = hs_setup(HSConfig(ni=64, nj=32, nk=10, dt=300, seed=0, uv_scheme=EPIC_UV_LEAPFROG))
    a, b = _pair(ga, f, prime=True)
    e = _run(a, b, DAY // 2)
    bounds = {"u": 5e-3, "v": 2e-3, "hdry": 1e-6, "theta": 1e-7}
    assert all(e[k][0] <= bounds[k] for k in bounds), e
    fa, fb = a.download(), b.download()
    assert (fa.struct.it_zero, fa.struct.itime) == (fb.struct.it_zero, fb.struct.itime)


def test_mixed_is_deterministic(gpu):
    """Two mixed runs (graph replay and single steps) give identical bits."""
    ga, f = hs_setup(HSConfig(ni=32, nj=16, nk=10, dt=300, seed=4))
    m1, m2 = Model(ga, EPIC_PREC_MIXED), Model(ga, EPIC_PREC_MIXED)
    for m in (m1, m2):
        m.upload(f)
        m.timestep(EPIC_SYNC_DIAGS_ONLY)
    m1.run(6)
    for _ in range(6):
        m2.run(1)
    m1.sync()
    m2.sync()
    a, b = m1.download(), m2.download()
    for k in a.arrays:
        assert np.array_equal(a.arrays[k], b.arrays[k]), k


def test_models_of_different_sizes_coexist(gpu):
    """Creating a smaller model after a larger one must not shrink any launch limit the larger
    one needs (shared-memory sizes depend on ni and nk)."""
    big_ga, big_f = hs_setup(HSConfig(ni=256, nj=128, nk=20, dt=150))
    big = Model(big_ga, EPIC_PREC_MIXED)
    big64 = Model(big_ga, EPIC_PREC_FP64)
    small_ga, small_f = hs_setup(HSConfig(ni=32, nj=16, nk=10, dt=300))
    small, small64 = Model(small_ga, EPIC_PREC_MIXED), Model(small_ga, EPIC_PREC_FP64)
    for m, f in ((big, big_f), (big64, big_f), (small, small_f), (small64, small_f)):
        m.upload(f)
        m.timestep(EPIC_SYNC_DIAGS_ONLY)
        m.run(2)
        m.sync()
