"""Batches (epic_batch_*): every kernel launched once for all members must give each member
exactly the bits it gets when stepped alone, in both precision forms."""
import numpy as np
import pytest

from epic_gb300 import (EPIC_ADV_AKIMA, EPIC_IO_ALL, EPIC_IO_STATE, EPIC_PREC_FP64, EPIC_PREC_MIXED, EPIC_PREC_MIXED_FAST, EPIC_PROFILE_N2,
                        EPIC_SYNC_DIAGS_ONLY, EPIC_UV_AB3, EPIC_UV_LEAPFROG, Batch, EpicError, HSConfig, Model, hs_setup)

pytestmark = pytest.mark.gpu


def _member(seed, kf_scale, precision, shape=(32, 16, 10), scheme=EPIC_UV_AB3, adv=0):
    ni, nj, nk = shape
    ga, f = hs_setup(HSConfig(ni=ni, nj=nj, nk=nk, dt=300, seed=seed, uv_scheme=scheme, advection_scheme=adv))
    ga.struct.hs_kf *= kf_scale
    m = Model(ga, precision)
    m.upload(f)
    return ga, f, m


@pytest.mark.parametrize("precision,scheme", [(EPIC_PREC_FP64, EPIC_UV_AB3), (EPIC_PREC_MIXED, EPIC_UV_AB3),
                                              (EPIC_PREC_MIXED_FAST, EPIC_UV_AB3), (EPIC_PREC_FP64, EPIC_UV_LEAPFROG),
                                              (EPIC_PREC_MIXED, EPIC_UV_LEAPFROG), (EPIC_PREC_MIXED_FAST, EPIC_UV_LEAPFROG)])
@pytest.mark.parametrize("adv", [0, EPIC_ADV_AKIMA])
def test_batch_equals_members_alone(gpu, precision, scheme, adv):
    scales = [1.0, 0.93, 1.07, 1.1, 0.9]
    members = [_member(10 + q, s, precision, scheme=scheme, adv=adv) for q, s in enumerate(scales)]
    batch = Batch([m for _, _, m in members])
    batch.timestep(EPIC_SYNC_DIAGS_ONLY)
    batch.run(7)
    batch.sync()
    for ga, f, m in members:
        alone = Model(ga, precision)
        alone.upload(f)
        alone.timestep(EPIC_SYNC_DIAGS_ONLY)
        alone.run(7)
        alone.sync()
        a, b = m.download(), alone.download()
        for k in a.arrays:
            assert np.array_equal(a.arrays[k], b.arrays[k]), k
        assert (a.struct.itime, a.struct.it_zero) == (b.struct.itime, b.struct.it_zero)
    assert batch.kernels_per_step > 0


@pytest.mark.parametrize("precision", [EPIC_PREC_FP64, EPIC_PREC_MIXED])
def test_gas_giant_batch_equals_members_alone(gpu, precision):
    """Jets over the gas-giant lower boundary (GZ_SURFACE from gz_from_u every store_pgrad_vars),
    members of two sizes in one batch: each equals itself stepped alone."""
    from epic_gb300 import EPIC_PROFILE_N2
    members = []
    for q, shape in enumerate([(32, 16, 10), (64, 32, 10), (32, 16, 10)]):
        ni, nj, nk = shape
        ga, f = hs_setup(HSConfig(ni=ni, nj=nj, nk=nk, dt=300, seed=40 + q, state="jet", profile=EPIC_PROFILE_N2, gas_giant=True))
        m = Model(ga, precision)
        m.upload(f)
        members.append((ga, f, m))
    batch = Batch([m for _, _, m in members])
    batch.timestep(EPIC_SYNC_DIAGS_ONLY)
    batch.run(5)
    batch.sync()
    for ga, f, m in members:
        alone = Model(ga, precision)
        alone.upload(f)
        alone.timestep(EPIC_SYNC_DIAGS_ONLY)
        alone.run(5)
        alone.sync()
        a, b = m.download(), alone.download()
        for k in a.arrays:
            assert np.array_equal(a.arrays[k], b.arrays[k]), k
        assert np.abs(a.arrays["gz_surface"]).max() > 0.


def test_batch_rejects_incompatible_members(gpu):
    """Members must share the layers, the precision form and, in the mixed forms, the zonal
    filter's path (tensor cores for ni a multiple of 128); ni, nj and dt may differ."""
    _, _, a = _member(1, 1.0, EPIC_PREC_FP64)
    _, _, b = _member(2, 1.0, EPIC_PREC_FP64, shape=(32, 16, 20))
    _, _, c = _member(3, 1.0, EPIC_PREC_MIXED)
    _, _, d = _member(4, 1.0, EPIC_PREC_MIXED_FAST)
    _, _, e = _member(5, 1.0, EPIC_PREC_MIXED, shape=(128, 64, 10))
    _, _, f = _member(6, 1.0, EPIC_PREC_FP64, shape=(64, 32, 10))
    with pytest.raises(EpicError, match="layers"):
        Batch([a, b])
    with pytest.raises(EpicError, match="precision"):
        Batch([a, c])
    with pytest.raises(EpicError, match="precision"):
        Batch([c, d])
    with pytest.raises(EpicError, match="filter path"):
        Batch([c, e])
    ga, fg = hs_setup(HSConfig(ni=32, nj=16, nk=10, dt=300, seed=7, gas_giant=True))
    g = Model(ga, EPIC_PREC_FP64)
    g.upload(fg)
    with pytest.raises(EpicError, match="lower boundary"):
        Batch([a, g])
    gh, fh = hs_setup(HSConfig(ni=32, nj=16, nk=10, dt=300, seed=7, x_h2=0.864, x_he=0.136))
    h = Model(gh, EPIC_PREC_FP64)
    h.upload(fh)
    with pytest.raises(EpicError, match="thermodynamics"):
        Batch([a, h])
    gt, ft = hs_setup(HSConfig(ni=32, nj=16, nk=10, dt=300, seed=7, turbulence=True))
    t1 = Model(gt, EPIC_PREC_FP64)
    t1.upload(ft)
    with pytest.raises(EpicError, match="turbulence"):
        Batch([a, t1])
    with pytest.raises(EpicError, match="turbulence"):   # the closure is in the FP64 form only
        Model(gt, EPIC_PREC_MIXED)
    Batch([a, f]).close()   # sizes alone may differ


@pytest.mark.parametrize("shapes", [[(32, 16, 300), (32, 16, 300), (32, 16, 150)], [(32, 16, 300), (64, 32, 300), (64, 48, 150)]],
                         ids=["same_size", "uneven"])
def test_turbulence_batch_equals_members_alone(gpu, shapes):
    """Three members with the turbulence closure (zonal jets, different seeds and time steps; of
    one size, or of different ni, nj, dt) in one batch: every member equals the same member
    stepped alone, bit for bit."""
    cfgs = [HSConfig(ni=ni, nj=nj, nk=10, dt=dt, seed=60 + q, state="jet", profile=EPIC_PROFILE_N2, turbulence=True)
            for q, (ni, nj, dt) in enumerate(shapes)]
    alone, models, fields = [], [], []
    for cfg in cfgs:
        ga, f = hs_setup(cfg)
        m = Model(ga, EPIC_PREC_FP64)
        m.upload(f)
        m.timestep(EPIC_SYNC_DIAGS_ONLY)
        m.run(5)
        m.sync()
        alone.append(m.download())
        b = Model(ga, EPIC_PREC_FP64)
        b.upload(f)
        models.append(b)
        fields.append(f)
    batch = Batch(models)
    batch.timestep(EPIC_SYNC_DIAGS_ONLY)
    batch.run(5)
    out = batch.download([f.copy() for f in fields])
    for q in range(3):
        for k in alone[q].arrays:
            assert np.array_equal(out[q].arrays[k], alone[q].arrays[k]), (q, k)


# Batches whose members differ in ni, nj and dt: one launch per kernel for all of them, each
# member's threads bounded by its own sizes, its pointers moved array by array.
UNEVEN = {
    "fp64": (EPIC_PREC_FP64, [(32, 16, 10, 300), (64, 32, 10, 300), (64, 48, 10, 150), (128, 64, 10, 150)]),
    "mixed_fft": (EPIC_PREC_MIXED, [(32, 16, 10, 300), (64, 32, 10, 300), (64, 40, 10, 150)]),
    "mixed_tensor": (EPIC_PREC_MIXED, [(128, 64, 20, 300), (256, 128, 20, 150), (128, 96, 20, 150)]),
    "fast_tensor": (EPIC_PREC_MIXED_FAST, [(128, 64, 20, 300), (256, 128, 20, 150)]),
}


def _uneven_member(q, shape, precision, scheme=EPIC_UV_AB3):
    ni, nj, nk, dt = shape
    ga, f = hs_setup(HSConfig(ni=ni, nj=nj, nk=nk, dt=dt, seed=200 + q, uv_scheme=scheme))
    ga.struct.hs_kf *= 1.0 + 0.03 * q
    m = Model(ga, precision)
    m.upload(f)
    return ga, f, m


@pytest.mark.parametrize("fused", [False, True], ids=["auto", "fused_march"])
@pytest.mark.parametrize("case", sorted(UNEVEN))
def test_uneven_batch_equals_members_alone(gpu, case, fused):
    from epic_gb300 import TUNE_HSU_MERID_VARIANT
    precision, shapes = UNEVEN[case]
    members = [_uneven_member(q, sh, precision) for q, sh in enumerate(shapes)]
    batch = Batch([m for _, _, m in members])
    if fused:
        table = [0] * (TUNE_HSU_MERID_VARIANT + 1)
        table[TUNE_HSU_MERID_VARIANT] = 1
        batch.set_tuning(table)
    batch.timestep(EPIC_SYNC_DIAGS_ONLY)
    batch.run(5)
    batch.sync()
    for q, (ga, f, m) in enumerate(members):
        alone = Model(ga, precision)
        alone.upload(f)
        alone.timestep(EPIC_SYNC_DIAGS_ONLY)
        alone.run(5)
        alone.sync()
        a, b = m.download(), alone.download()
        for k in a.arrays:
            assert np.array_equal(a.arrays[k], b.arrays[k]), (shapes[q], k)
        assert (a.struct.itime, a.struct.it_zero, a.struct.model_time) == (b.struct.itime, b.struct.it_zero, b.struct.model_time)


def test_uneven_batch_leapfrog_and_pipeline(gpu):
    """Leapfrog members of three sizes through the pipelined end-to-end step (sub-batches of
    uneven members on their own streams)."""
    shapes = [(32, 16, 10, 300), (64, 32, 10, 300), (64, 24, 10, 150)]
    members = [_uneven_member(q, sh, EPIC_PREC_MIXED, EPIC_UV_LEAPFROG) for q, sh in enumerate(shapes)]
    b = Batch([m for _, _, m in members])
    b.timestep(EPIC_SYNC_DIAGS_ONLY)
    b.sync()
    hosts = [m.download().copy(pinned=True) for _, _, m in members]
    b.step_host(hosts, 3, groups=2)
    for (ga, f, _), h in zip(members, hosts):
        alone = Model(ga, EPIC_PREC_MIXED)
        alone.upload(f)
        alone.timestep(EPIC_SYNC_DIAGS_ONLY)
        alone.run(3)
        alone.sync()
        w = alone.download()
        for k in w.arrays:
            assert np.array_equal(h.arrays[k], w.arrays[k]), k


def test_autotuned_shapes_change_no_result(gpu):
    """Tuning picks block sizes only; a tuned batch gives the bits of the untuned one."""
    members = [_member(20 + q, 1.0, EPIC_PREC_MIXED) for q in range(3)]
    scratch = Batch([m for _, _, m in members])
    scratch.timestep(EPIC_SYNC_DIAGS_ONLY)
    table = scratch.autotune(trial_steps=1)
    scratch.close()
    assert len(table) == 10 and all(t > 0 for t in table)
    tuned = [_member(30 + q, 1.0, EPIC_PREC_MIXED) for q in range(3)]
    plain = [_member(30 + q, 1.0, EPIC_PREC_MIXED) for q in range(3)]
    bt, bp = Batch([m for _, _, m in tuned]), Batch([m for _, _, m in plain])
    bt.set_tuning([64, 256, 512, 64, 256, 512, 64, 512, 32, 1])
    for b in (bt, bp):
        b.timestep(EPIC_SYNC_DIAGS_ONLY)
        b.run(4)
        b.sync()
    for (_, _, a), (_, _, c) in zip(tuned, plain):
        x, y = a.download(), c.download()
        for k in x.arrays:
            assert np.array_equal(x.arrays[k], y.arrays[k]), k


def test_batch_upload_download_match_members(gpu):
    """epic_batch_upload/download move every member's state like the per-member calls."""
    members = [_member(40 + q, 1.0 + 0.05 * q, EPIC_PREC_FP64) for q in range(3)]
    b = Batch([m for _, _, m in members])
    b.upload([f for _, f, _ in members])
    b.timestep(EPIC_SYNC_DIAGS_ONLY)
    b.run(3)
    b.sync()
    got = b.download([m.download().copy() for _, _, m in members])
    for (ga, f, m), g in zip(members, got):
        alone = Model(ga, EPIC_PREC_FP64)
        alone.upload(f)
        alone.timestep(EPIC_SYNC_DIAGS_ONLY)
        alone.run(3)
        alone.sync()
        w = alone.download()
        for k in w.arrays:
            assert np.array_equal(g.arrays[k], w.arrays[k]), k
        assert g.struct.itime == w.struct.itime


PROGNOSTIC = ("u", "v", "dudt", "dvdt", "hdry", "theta")


@pytest.mark.parametrize("io", [EPIC_IO_ALL, EPIC_IO_STATE], ids=["all", "state"])
@pytest.mark.parametrize("groups", [1, 2, 3])
def test_batch_step_host_pipeline(gpu, groups, io):
    """The pipelined end-to-end step (host-resident state, sub-batches on their own streams)
    gives every member the bits it gets stepped alone: every array with EPIC_IO_ALL; with
    EPIC_IO_STATE the prognostic arrays that move each step, and the diagnostics left on the
    device once they are downloaded."""
    members = [_member(60 + q, 1.0 - 0.04 * q, EPIC_PREC_MIXED) for q in range(3)]
    b = Batch([m for _, _, m in members])
    b.timestep(EPIC_SYNC_DIAGS_ONLY)
    b.sync()
    hosts = [m.download().copy(pinned=True) for _, _, m in members]
    b.step_host(hosts, 4, groups=groups, io=io)
    diags = [m.download() for _, _, m in members]
    for (ga, f, _), h, dg in zip(members, hosts, diags):
        alone = Model(ga, EPIC_PREC_MIXED)
        alone.upload(f)
        alone.timestep(EPIC_SYNC_DIAGS_ONLY)
        alone.run(4)
        alone.sync()
        w = alone.download()
        for k in w.arrays:
            got = h.arrays[k] if io == EPIC_IO_ALL or k in PROGNOSTIC else dg.arrays[k]
            assert np.array_equal(got, w.arrays[k]), (groups, k)
        assert h.struct.itime == w.struct.itime


@pytest.mark.parametrize("io", [EPIC_IO_ALL, EPIC_IO_STATE], ids=["all", "state"])
def test_turbulence_step_host_pipeline(gpu, io):
    """The pipelined end-to-end step with the turbulence closure: NU_TURB moves with the
    prognostic arrays (EPIC_IO_STATE), the diffusivities stay on the device; every member equals
    the same member stepped alone, bit for bit."""
    cfgs = [HSConfig(ni=32, nj=16, nk=10, dt=300, seed=70 + q, state="jet", profile=EPIC_PROFILE_N2, turbulence=True)
            for q in range(3)]
    members = []
    for cfg in cfgs:
        ga, f = hs_setup(cfg)
        m = Model(ga, EPIC_PREC_FP64)
        m.upload(f)
        members.append((ga, f, m))
    b = Batch([m for _, _, m in members])
    b.timestep(EPIC_SYNC_DIAGS_ONLY)
    b.sync()
    hosts = [m.download().copy(pinned=True) for _, _, m in members]
    b.step_host(hosts, 3, groups=2, io=io)
    diags = [m.download() for _, _, m in members]
    for (ga, f, _), h, dg in zip(members, hosts, diags):
        alone = Model(ga, EPIC_PREC_FP64)
        alone.upload(f)
        alone.timestep(EPIC_SYNC_DIAGS_ONLY)
        alone.run(3)
        alone.sync()
        w = alone.download()
        for k in w.arrays:
            got = h.arrays[k] if io == EPIC_IO_ALL or k in PROGNOSTIC + ("nu_turb",) else dg.arrays[k]
            assert np.array_equal(got, w.arrays[k]), (io, k)


def test_state_io_needs_uploaded_members(gpu):
    """EPIC_IO_STATE moves the prognostic arrays only, so it refuses members with no state."""
    ga, f = hs_setup(HSConfig(ni=32, nj=16, nk=10, dt=300, seed=3))
    fresh = Model(ga, EPIC_PREC_MIXED)
    b = Batch([fresh])
    with pytest.raises(EpicError, match="no state on the device"):
        b.step_host([f.copy(pinned=True)], 1, groups=1, io=EPIC_IO_STATE)


# 26 members of 128x64x20: the UNITY and HDRY passes of the meridional Hsu advection cover
# 128 * 20 * 26 = 66,560 (k, i, member) columns, past the 65,536 at which the batch launch takes
# the fused march (k_hsu_meridional), as the 64-member ensemble of the benchmark does; THETA's
# pass (k >= k_sigma - 1, two layers) stays on the four passes, as it does there.  A model stepped
# alone takes the four passes for all three.
FUSED_MEMBERS = 26


@pytest.mark.parametrize("precision", [EPIC_PREC_FP64, EPIC_PREC_MIXED, EPIC_PREC_MIXED_FAST])
def test_fused_meridional_march_batch_equals_members_alone(gpu, precision):
    from oracle_lib import Port
    shape = (128, 64, 20)
    assert shape[0] * shape[2] * FUSED_MEMBERS >= 65536
    members = [_member(100 + q, 1.0 + 0.1 * ((q * 7) % 11 - 5) / 5, precision, shape=shape) for q in range(FUSED_MEMBERS)]
    batch = Batch([m for _, _, m in members])
    batch.timestep(EPIC_SYNC_DIAGS_ONLY)
    batch.run(3)
    batch.sync()
    for q, (ga, f, m) in enumerate(members):
        alone = Model(ga, precision)
        alone.upload(f)
        alone.timestep(EPIC_SYNC_DIAGS_ONLY)
        alone.run(3)
        alone.sync()
        a, b = m.download(), alone.download()
        for k in a.arrays:
            assert np.array_equal(a.arrays[k], b.arrays[k]), (q, k)
        alone.close()
    if precision == EPIC_PREC_FP64:
        # and the batch's first member is the oracle's grid bit for bit
        ga, f, m = members[0]
        port = Port(ga, cr_libm=True)
        port.upload(f)
        port.timestep(EPIC_SYNC_DIAGS_ONLY)
        port.run(3)
        a, b = m.download(), port.download()
        for k in a.arrays:
            assert np.array_equal(a.arrays[k], b.arrays[k]), k
    batch.close()
    for _, _, m in members:
        m.close()


def test_divergence_damping_batch_equals_members_alone(gpu):
    """nudiv > 0 (divergence_damping runs in every step) in a mixed batch of three members."""
    members = []
    for q in range(3):
        ga, f = hs_setup(HSConfig(ni=32, nj=16, nk=10, dt=300, seed=70 + q, nudiv=0.5))
        m = Model(ga, EPIC_PREC_MIXED)
        m.upload(f)
        members.append((ga, f, m))
    b = Batch([m for _, _, m in members])
    b.timestep(EPIC_SYNC_DIAGS_ONLY)
    b.run(5)
    b.sync()
    for ga, f, m in members:
        alone = Model(ga, EPIC_PREC_MIXED)
        alone.upload(f)
        alone.timestep(EPIC_SYNC_DIAGS_ONLY)
        alone.run(5)
        alone.sync()
        x, y = m.download(), alone.download()
        for k in x.arrays:
            assert np.array_equal(x.arrays[k], y.arrays[k]), k


def test_batch_members_on_one_device(gpu):
    """Models record the device they were created on; a batch of them is created on it.  (A batch
    mixing devices is refused with EPIC_ERR_ARG; one GPU cannot show that case.)"""
    import torch
    members = [_member(80 + q, 1.0, EPIC_PREC_FP64) for q in range(2)]
    assert all(m.device == torch.cuda.current_device() for _, _, m in members)
    b = Batch([m for _, _, m in members])
    b.timestep(EPIC_SYNC_DIAGS_ONLY)
    b.sync()


@pytest.mark.parametrize("shape", [(32, 16, 10), (128, 64, 10)], ids=["fft_filter", "tensor_filter"])
def test_halted_member_stops_and_reports(gpu, shape):
    """A member whose state makes the reference stop (a negative potential temperature in one cell:
    GZ3 not monotonic in store_pgrad_vars, found by the priming call) halts after the step in which
    the error is seen: its state and itime stop changing and every sync reports it, while the other
    member of the batch keeps stepping (at 128 x 64 the two share the tensor-core filter's CTAs,
    which must leave the halted member's planes alone)."""
    from epic_gb300 import Fields
    members = [_member(90 + q, 1.0, EPIC_PREC_MIXED, shape=shape) for q in range(2)]
    ga, f, bad = members[1]
    broken = f.copy()
    broken.theta[10, 5, 5] = -1.0
    bad.upload(broken)
    b = Batch([m for _, _, m in members])
    b.timestep(EPIC_SYNC_DIAGS_ONLY)
    b.run(3)
    with pytest.raises(EpicError, match="member 1: store_pgrad_vars: GZ3 not monotonic"):
        b.sync()
    good = members[0][2]
    g0 = good.download()
    h0 = Fields(*shape, f.uv_scheme)
    with pytest.raises(EpicError, match="GZ3 not monotonic"):
        bad.download(h0)
    b.run(2)
    with pytest.raises(EpicError, match="member 1"):
        b.sync()
    g1 = good.download()
    h1 = Fields(*shape, f.uv_scheme)
    with pytest.raises(EpicError):
        bad.download(h1)
    assert g1.struct.itime == g0.struct.itime + 2
    assert h1.struct.itime == h0.struct.itime
    for k in h0.arrays:
        assert np.array_equal(h0.arrays[k], h1.arrays[k], equal_nan=True), k
