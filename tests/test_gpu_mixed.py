"""The two mixed-precision forms against the FP64 form on the GPU.

EPIC_PREC_MIXED: stencils, advection, hyperviscosity, the zonal filter (on the tensor cores for
ni a multiple of 128), calc_w and the physics evaluate in FP32; the vertical pressure and
geopotential integration (set_p2etc, store_pgrad_vars), the pressure gradient, the running sums,
every update of a stored field and the Adams-Bashforth/leapfrog step stay FP64 (the state is
stored in FP64).
EPIC_PREC_MIXED_FAST: the same with set_p2etc, store_pgrad_vars and the pressure gradient in FP32
too (their running sums and the updates stay FP64).

Stated error (relative L2 per field vs FP64, dt 300 s), measured on a GB300:

  form   shape      case                              U        V        HDRY     THETA
  mixed  64x32x10   1 day after a 10-day spin-up      6.1e-6   2.1e-5   3.1e-8   3.1e-10
  mixed  64x32x10   1 day from rest                   3.9e-5   2.5e-5   2.4e-8   2.0e-10
  mixed  64x32x10   12 h from rest, leapfrog          5.8e-4   1.4e-4   3.7e-8   9.5e-11
  mixed  128x64x20  1 day after a 1-day spin-up       3.8e-5   2.3e-5   1.7e-7   8.4e-10
  mixed  128x64x20  1 day from rest                   1.0e-4   1.3e-4   1.6e-6   8.3e-9
  fast   64x32x10   1 day after a 10-day spin-up      3.7e-5   6.0e-4   3.8e-7   3.7e-8
  fast   64x32x10   1 day from rest                   2.5e-4   8.7e-4   2.1e-7   3.7e-8
  fast   64x32x10   12 h from rest, leapfrog          1.8e-3   6.4e-4   1.6e-7   3.7e-8
  fast   128x64x20  1 day after a 1-day spin-up       3.4e-4   9.7e-4   1.1e-5   7.0e-8
  fast   128x64x20  1 day from rest                   9.5e-4   1.7e-3   2.0e-5   1.2e-7
  mixed  64x32x10   zonal jets, 1 day                 3.4e-7   8.9e-7   1.7e-8   3.4e-9
  fast   64x32x10   zonal jets, 1 day                 3.6e-6   1.8e-5   1.4e-7   3.8e-8
  mixed  64x32x10   jets, gas-giant boundary, 1 day   3.7e-7   7.3e-7   1.1e-7   4.1e-9
  mixed  64x32x10   same with hydrogen, dt 150, 1 day 3.6e-7   6.8e-7   1.6e-7   3.8e-9
  fast   64x32x10   same with hydrogen, dt 150, 1 day 3.5e-6   5.6e-6   2.6e-7   3.7e-8

(128x64x20 is the ensemble member shape: ni = 128 takes the tensor-core filter; its FP64 run
stays stable for about two days, so its spin-up is one day.)

The first hours from rest are driven by horizontal pressure differences 1e-5 of the geopotential,
so rounding is amplified there (the leapfrog case ends at 12 h: the FP64 leapfrog run of this
configuration itself stops with non-monotonic GZ3 in its second day).  The fast form's V error
comes from FP32 rounding of P2, THETA and GZ3 recomputed every step (the pressure-gradient
chain); the mixed form keeps that chain in double-float and stays within 1e-4 after one day but for the
first day from rest at 128x64x20.  The pressure gradient amplifies rounding in its inputs
(GZ3, P2, RHO3 differ by ~1e-5 of their size across a cell), so every FP32 rounding of a state
field or of a quantity the vertical integration reads (W3 from calc_w, the hyperviscous
increments, the 3-D filter's profile) shows up in the winds; the mixed form takes those in
binary64 or as FP32 increments on binary64 values.  The bounds below leave a factor ~3 over the
figures.
"""
import numpy as np
import pytest

from compare import PROGNOSTIC, field_errors
from epic_gb300 import (EPIC_ADV_AKIMA, EPIC_ADV_HSU, EPIC_PREC_FP64, EPIC_PREC_MIXED, EPIC_PREC_MIXED_FAST,
                        EPIC_PROFILE_N2, EPIC_SYNC_DIAGS_ONLY, EPIC_UV_LEAPFROG, HSConfig, Model, hs_setup)

pytestmark = pytest.mark.gpu
DAY = 288   # steps of 300 s
FORMS = {"mixed": EPIC_PREC_MIXED, "fast": EPIC_PREC_MIXED_FAST}
BOUNDS = {
    ("mixed", "spun_up"): {"u": 2e-5, "v": 8e-5, "hdry": 1e-7, "theta": 1e-9},
    ("mixed", "rest"): {"u": 1.2e-4, "v": 8e-5, "hdry": 1e-7, "theta": 1e-9},
    ("mixed", "leapfrog"): {"u": 2e-3, "v": 5e-4, "hdry": 1.2e-7, "theta": 5e-10},
    ("mixed", "member_spun_up"): {"u": 1.2e-4, "v": 8e-5, "hdry": 6e-7, "theta": 3e-9},
    ("mixed", "member_rest"): {"u": 1e-4, "v": 1e-4, "hdry": 1e-4, "theta": 1e-4},   # the benchmark spec bound
    ("fast", "member_spun_up"): {"u": 1e-3, "v": 3e-3, "hdry": 3.5e-5, "theta": 2e-7},
    ("fast", "member_rest"): {"u": 3e-3, "v": 5e-3, "hdry": 6e-5, "theta": 4e-7},
    ("mixed", "jet"): {"u": 1.2e-6, "v": 3e-6, "hdry": 6e-8, "theta": 1e-8},
    ("fast", "jet"): {"u": 1.2e-5, "v": 6e-5, "hdry": 5e-7, "theta": 1.2e-7},
    # the jets over the gas-giant lower boundary: GZ_SURFACE follows the bottom wind, whose
    # rounding then moves the whole column (mixed, measured: U 3.7e-7, V 7.3e-7, HDRY 1.1e-7,
    # THETA 4.1e-9)
    ("mixed", "jet-gg"): {"u": 8e-7, "v": 1.5e-6, "hdry": 2.2e-7, "theta": 1e-8},
    ("fast", "jet-gg"): {"u": 1.2e-5, "v": 6e-5, "hdry": 2e-6, "theta": 1.2e-7},
    # the same with the hydrogen-helium thermodynamics, dt 150 (measured: mixed U 3.6e-7, V 6.8e-7,
    # HDRY 1.6e-7, THETA 3.8e-9; fast U 3.5e-6, V 5.6e-6, HDRY 2.6e-7, THETA 3.7e-8)
    ("mixed", "jet-gg-h2"): {"u": 8e-7, "v": 1.5e-6, "hdry": 3.5e-7, "theta": 1e-8},
    ("fast", "jet-gg-h2"): {"u": 8e-6, "v": 1.5e-5, "hdry": 6e-7, "theta": 8e-8},
    ("fast", "spun_up"): {"u": 1e-4, "v": 2e-3, "hdry": 1e-6, "theta": 1e-7},
    ("fast", "rest"): {"u": 1e-3, "v": 3e-3, "hdry": 1e-6, "theta": 1e-7},
    ("fast", "leapfrog"): {"u": 6e-3, "v": 3e-3, "hdry": 1e-6, "theta": 1e-7},
}


@pytest.fixture(scope="module")
def spun_up(gpu):
    ga, f = hs_setup(HSConfig(ni=64, nj=32, nk=10, dt=300, seed=0))
    m = Model(ga, EPIC_PREC_FP64)
    m.upload(f)
    m.timestep(EPIC_SYNC_DIAGS_ONLY)
    m.run(10 * DAY)
    m.sync()
    return ga, m.download()


def _pair(ga, f, prime, precision):
    a, b = Model(ga, EPIC_PREC_FP64), Model(ga, precision)
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


def _check(e, bounds):
    assert all(e[k][0] <= bounds[k] for k in bounds), e


@pytest.mark.parametrize("form", FORMS)
def test_one_day_after_spin_up(spun_up, form):
    ga, f = spun_up
    a, b = _pair(ga, f, False, FORMS[form])
    _check(_run(a, b, DAY), BOUNDS[(form, "spun_up")])


@pytest.mark.parametrize("form", FORMS)
def test_one_day_from_rest(gpu, form):
    ga, f = hs_setup(HSConfig(ni=64, nj=32, nk=10, dt=300, seed=0))
    a, b = _pair(ga, f, True, FORMS[form])
    _check(_run(a, b, DAY), BOUNDS[(form, "rest")])


@pytest.mark.parametrize("form", FORMS)
def test_leapfrog_follows_fp64(gpu, form):
    """The leapfrog (Asselin-filtered) wind step, 12 simulated hours from rest; the time-plane
    bookkeeping (IT_ZERO, itime) must be the FP64 form's."""
    ga, f = hs_setup(HSConfig(ni=64, nj=32, nk=10, dt=300, seed=0, uv_scheme=EPIC_UV_LEAPFROG))
    a, b = _pair(ga, f, True, FORMS[form])
    _check(_run(a, b, DAY // 2), BOUNDS[(form, "leapfrog")])
    fa, fb = a.download(), b.download()
    assert (fa.struct.it_zero, fa.struct.itime) == (fb.struct.it_zero, fb.struct.itime)


@pytest.mark.parametrize("form", FORMS)
def test_is_deterministic(gpu, form):
    """Two runs (graph replay and single steps) give identical bits."""
    ga, f = hs_setup(HSConfig(ni=32, nj=16, nk=10, dt=300, seed=4))
    m1, m2 = Model(ga, FORMS[form]), Model(ga, FORMS[form])
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
    small_ga, small_f = hs_setup(HSConfig(ni=32, nj=16, nk=10, dt=300))
    models = []
    for prec in (EPIC_PREC_MIXED, EPIC_PREC_MIXED_FAST, EPIC_PREC_FP64):
        models.append((Model(big_ga, prec), big_f))
    for prec in (EPIC_PREC_MIXED, EPIC_PREC_MIXED_FAST, EPIC_PREC_FP64):
        models.append((Model(small_ga, prec), small_f))
    for m, f in models:
        m.upload(f)
        m.timestep(EPIC_SYNC_DIAGS_ONLY)
        m.run(2)
        m.sync()


@pytest.mark.parametrize("form", FORMS)
def test_akima_one_day_after_spin_up(spun_up, form):
    """The Akima advection scheme, one day from the spun-up state (the state's winds and mass
    come from the Hsu-scheme spin-up; the day is stepped with Akima in both forms)."""
    ga, f = spun_up
    ga.struct.advection_scheme = EPIC_ADV_AKIMA
    try:
        a, b = _pair(ga, f, False, FORMS[form])
    finally:
        ga.struct.advection_scheme = EPIC_ADV_HSU
    _check(_run(a, b, DAY), BOUNDS[(form, "spun_up")])


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("case", ["member_spun_up", "member_rest"])
def test_one_day_at_member_shape(gpu, form, case):
    """The ensemble member shape 128x64x20 (tensor-core filter, 20 layers), one day from rest or
    after a one-day FP64 spin-up."""
    ga, f = hs_setup(HSConfig(ni=128, nj=64, nk=20, dt=300, seed=0))
    prime = case == "member_rest"
    if not prime:
        m = Model(ga, EPIC_PREC_FP64)
        m.upload(f)
        m.timestep(EPIC_SYNC_DIAGS_ONLY)
        m.run(DAY)
        m.sync()
        f = m.download()
    a, b = _pair(ga, f, prime, FORMS[form])
    _check(_run(a, b, DAY), BOUNDS[(form, case)])


@pytest.mark.parametrize("gas_giant", [False, True], ids=["terrain", "gas_giant"])
@pytest.mark.parametrize("form", FORMS)
def test_jets_one_day(gpu, form, gas_giant):
    """The balanced zonal-jet state on the constant-N^2 sounding, one day; over the terrestrial
    and over the gas-giant lower boundary (GZ_SURFACE from gz_from_u, binary64 in every form)."""
    ga, f = hs_setup(HSConfig(ni=64, nj=32, nk=10, dt=300, seed=0, profile=EPIC_PROFILE_N2, state="jet", gas_giant=gas_giant))
    a, b = _pair(ga, f, True, FORMS[form])
    _check(_run(a, b, DAY), BOUNDS[(form, "jet-gg" if gas_giant else "jet")])


@pytest.mark.parametrize("form", FORMS)
def test_hydrogen_jets_one_day(gpu, form):
    """The zonal jets over the gas-giant lower boundary with the hydrogen-helium thermodynamics
    (x_h2 = 0.864, x_he = 0.136: T3, T2 and the enthalpy of MONT3 from thermo_setup's tables, in
    binary64 in every form), one day against the FP64 form; dt 150 s (at dt 300 s the FP64 step,
    as the reference's, stops with non-monotonic GZ3 after 250 steps)."""
    ga, f = hs_setup(HSConfig(ni=64, nj=32, nk=10, dt=150, seed=0, profile=EPIC_PROFILE_N2, state="jet", gas_giant=True,
                              x_h2=0.864, x_he=0.136))
    a, b = _pair(ga, f, True, FORMS[form])
    e = _run(a, b, 2 * DAY)
    print(form, "jet-gg-h2", {k: float(v[0]) for k, v in e.items()})
    _check(e, BOUNDS[(form, "jet-gg-h2")])


@pytest.mark.parametrize("shape,dt,steps", [((256, 128, 10), 120, 240), ((512, 256, 10), 60, 120)])
def test_wide_grids_follow_fp64(gpu, shape, dt, steps):
    """Single models wide enough for two and four 128-point output tiles per row of the
    tensor-core filter (whose launcher spreads a row's tiles over several CTAs when only a few
    members fill the GPU, for calls that do not filter in place): the mixed form stays near FP64
    over hours, and repeats itself bit for bit."""
    ni, nj, nk = shape
    ga, f = hs_setup(HSConfig(ni=ni, nj=nj, nk=nk, dt=dt, seed=2))
    a, b = _pair(ga, f, True, EPIC_PREC_MIXED)
    _check(_run(a, b, steps), {"u": 2e-4, "v": 2e-4, "hdry": 1e-6, "theta": 1e-8})
    c = Model(ga, EPIC_PREC_MIXED)
    c.upload(f)
    c.timestep(EPIC_SYNC_DIAGS_ONLY)
    c.run(steps)
    c.sync()
    x, y = b.download(), c.download()
    for k in x.arrays:
        assert np.array_equal(x.arrays[k], y.arrays[k]), k


# The mixed form's error bound of the configuration: relative L2 <= 1e-4 per prognostic after one
# simulated day, for every member of the ensemble (measured over the members' interior cells).
NORTH_STAR_BOUND = 1e-4


def test_every_ensemble_member_within_bound(gpu):
    """Sixteen members of the 128x64x20 ensemble (noise seed q, drag rate k_f scaled by the
    benchmark's seeded factors), stepped one simulated day from rest as a batch in FP64 and in
    EPIC_PREC_MIXED: every member's U, V, HDRY and THETA within NORTH_STAR_BOUND of its FP64 run."""
    from epic_gb300 import Batch
    from epic_gb300.abi import Layout
    rng = np.random.default_rng(7)
    scales = [1.0 + float(rng.uniform(-0.1, 0.1)) for _ in range(16)]
    runs = {}
    for prec in (EPIC_PREC_FP64, EPIC_PREC_MIXED):
        members = []
        for q, sc in enumerate(scales):
            ga, f = hs_setup(HSConfig(ni=128, nj=64, nk=20, dt=300, seed=q))
            ga.struct.hs_kf *= sc
            m = Model(ga, prec)
            m.upload(f)
            members.append(m)
        b = Batch(members)
        b.timestep(EPIC_SYNC_DIAGS_ONLY)
        b.run(DAY)
        b.sync()
        runs[prec] = [m.download() for m in members]
        b.close()
    L = Layout(128, 64, 20)
    kinds = {"u": "uv", "v": "vv", "hdry": "h", "theta": "h"}
    worst = {}
    for k, kind in kinds.items():
        pick = (lambda f: f.wind(k)) if k in ("u", "v") else (lambda f: f.arrays[k])
        errs = []
        for got, ref in zip(runs[EPIC_PREC_MIXED], runs[EPIC_PREC_FP64]):
            a, r = L.interior(pick(got), kind), L.interior(pick(ref), kind)
            errs.append(float(np.linalg.norm(a - r) / np.linalg.norm(r)))
        worst[k] = max(errs)
    assert all(v <= NORTH_STAR_BOUND for v in worst.values()), worst
