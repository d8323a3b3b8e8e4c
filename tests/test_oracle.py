"""The oracle: its CPU restatement against the reference build and the golden fixtures.

* test_restatement_matches_reference: the restatement (oracle/epic_port.c) reproduces the
  reference's own step (oracle/_ref, compiled from the reference sources) bit for bit.  Runs
  only where the reference tree is present.
* test_golden_*: the restatement, from the inputs stored in tests/golden/*.npz, against the
  reference outputs stored there.  Runs everywhere (the fixtures were made by
  tests/golden/make_golden.py from the reference build).
"""
import glob
import os

import numpy as np
import pytest

from compare import PROGNOSTIC, field_errors
from epic_gb300 import (EPIC_ADV_AKIMA, EPIC_ADV_HSU, EPIC_PROFILE_N2, EPIC_SYNC_DIAGS_ONLY, EPIC_UV_AB3, EPIC_UV_LEAPFROG,
                        Fields, GridArrays, HSConfig, hs_setup)
from oracle_lib import Port, dict_to_fields, fields_to_dict, reference_available, run_reference

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))


def grid_from_fixture(z) -> GridArrays:
    ni, nj, nk = int(z["scalar_ni"]), int(z["scalar_nj"]), int(z["scalar_nk"])
    ga = GridArrays(ni, nj, nk)
    for k in ga.arrays:
        ga.arrays[k][...] = z["grid_" + k]
    for name in z.files:
        if name.startswith("scalar_"):
            key = name[len("scalar_"):]
            v = z[name]
            if key == "nu":
                for i in range(9):
                    ga.struct.nu[i] = float(v[i])
            else:
                setattr(ga.struct, key, v.item())
    return ga


def inputs_from_fixture(z, ga) -> Fields:
    turb = "in_nu_turb" in z.files   # fixtures of the turbulence closure
    f = Fields(ga.layout.ni, ga.layout.nj, ga.layout.nk, int(z["scalar_uv_scheme"]), turbulence=turb)
    for k in ("u", "v", "dudt", "dvdt", "hdry", "theta", "p3", "gz_surface", "u_spinup") + (("nu_turb",) if turb else ()):
        f.arrays[k][...] = z["in_" + k]
    for n in ("it_zero", "it_minus1", "it_minus2", "itime", "model_time"):
        setattr(f.struct, n, int(z["in_" + n]))
    return f


def snapshots(z):
    tags = sorted({n.split("_")[0] for n in z.files if n.startswith(("sync_", "step"))},
                  key=lambda t: -1 if t == "sync" else int(t[4:]))
    return tags


def compare_snapshot(f: Fields, z, tag, tol):
    bad = {}
    extra = ("gz_surface",) if f"{tag}_gz_surface" in z.files else ()   # fixtures of the gas-giant boundary
    extra += tuple(k for k in ("nu_turb", "diffusion_coef_theta", "diffusion_coef_uv") if f"{tag}_{k}" in z.files)
    for k in ("u", "v", "hdry", "theta", "p3", "gz3", "pv3", "w3", "heat3", "div_uv3") + extra:
        want = z[f"{tag}_{k}"]
        got = f.arrays[k]
        big = np.abs(want) > 1e300
        assert np.array_equal(np.abs(got) > 1e300, big), (tag, k)
        w, g = np.where(big, 0., want), np.where(big, 0., got)
        den = np.linalg.norm(w)
        rel = np.linalg.norm(g - w) / den if den > 0 else np.linalg.norm(g - w)
        if rel > tol:
            bad[k] = rel
    for n in ("it_zero", "it_minus1", "it_minus2", "model_time"):
        assert int(getattr(f.struct, n)) == int(z[f"{tag}_{n}"]), (tag, n)
    return bad


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def test_golden_restatement(path):
    """Restatement vs the reference's outputs stored in the fixture (1e-13: identical bits on
    x86-64; aarch64 glibc may round a few log/exp/pow results differently)."""
    z = np.load(path)
    ga = grid_from_fixture(z)
    f = inputs_from_fixture(z, ga)
    port = Port(ga)
    port.upload(f)
    done = 0
    for tag in snapshots(z):
        if tag == "sync":
            port.timestep(EPIC_SYNC_DIAGS_ONLY)
        else:
            n = int(tag[4:])
            port.run(n - done)
            done = n
        bad = compare_snapshot(port.download(), z, tag, 1e-13)
        assert not bad, (tag, bad)


def test_golden_inputs_match_generator():
    """The committed inputs equal what epic_hs_grid_build/epic_hs_initial_state produce now."""
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "hs32x16x10_ab3.npz"))   # seed 11
    ga0 = grid_from_fixture(z)
    s = ga0.struct
    cfg = HSConfig(ni=s.ni, nj=s.nj, nk=s.nk, dt=s.dt, uv_scheme=s.uv_scheme, seed=11)
    ga, f = hs_setup(cfg)
    for k in ga.arrays:
        np.testing.assert_allclose(ga.arrays[k], ga0.arrays[k], rtol=1e-14, atol=0, err_msg=k)
    np.testing.assert_allclose(f.arrays["p3"], z["in_p3"], rtol=1e-13, atol=0)
    np.testing.assert_allclose(f.arrays["theta"], z["in_theta"], rtol=1e-13, atol=0)


@pytest.mark.reference
@pytest.mark.parametrize("scheme,shape,steps,adv,state", [(EPIC_UV_AB3, (64, 32, 10), 12, EPIC_ADV_HSU, "hs"),
                                                           (EPIC_UV_LEAPFROG, (32, 16, 10), 6, EPIC_ADV_HSU, "hs"),
                                                           (EPIC_UV_AB3, (32, 16, 20), 4, EPIC_ADV_HSU, "hs"),
                                                           (EPIC_UV_AB3, (64, 32, 10), 12, EPIC_ADV_AKIMA, "hs"),
                                                           (EPIC_UV_LEAPFROG, (32, 16, 10), 6, EPIC_ADV_AKIMA, "hs"),
                                                           (EPIC_UV_AB3, (64, 32, 10), 12, EPIC_ADV_HSU, "jet"),
                                                           (EPIC_UV_LEAPFROG, (32, 16, 10), 6, EPIC_ADV_HSU, "jet"),
                                                           (EPIC_UV_AB3, (64, 32, 10), 12, EPIC_ADV_HSU, "jet-gas-giant"),
                                                           (EPIC_UV_LEAPFROG, (32, 16, 10), 6, EPIC_ADV_HSU, "hs-gas-giant")])
def test_restatement_matches_reference(scheme, shape, steps, adv, state):
    """The restatement against the reference's own step, every field bit for bit after every step;
    the "-gas-giant" states run with planet->type "gas-giant" (GZ_SURFACE from gz_from_u)."""
    if not reference_available():
        pytest.skip("reference source tree not present on this host")
    ni, nj, nk = shape
    gas_giant = state.endswith("-gas-giant")
    state = state.replace("-gas-giant", "")
    cfg = HSConfig(ni=ni, nj=nj, nk=nk, dt=300, uv_scheme=scheme, seed=5, advection_scheme=adv, state=state,
                   profile=EPIC_PROFILE_N2 if state == "jet" else 0, gas_giant=gas_giant)
    ga, f = hs_setup(cfg)
    sched = [("sync", 0)] + [("step", 1)] * steps
    geo, snaps = run_reference(ga, f, sched)
    assert max(geo) == 0.0, "grid geometry differs from the reference's set_lonlat/set_fmn/set_gravity/set_dsgth"
    port = Port(ga)
    port.upload(f)
    for i, (what, n) in enumerate(sched):
        if what == "sync":
            port.timestep(EPIC_SYNC_DIAGS_ONLY)
        else:
            port.run(n)
        got = port.download()
        want = dict_to_fields(snaps[i], ni, nj, nk, scheme)
        for k in got.arrays:
            assert np.array_equal(got.arrays[k], want.arrays[k]), f"snapshot {i}: field {k} differs"
        assert fields_to_dict(got)["it_zero"] == snaps[i]["it_zero"]


@pytest.mark.reference
@pytest.mark.parametrize("scheme,state", [(EPIC_UV_AB3, "hs"), (EPIC_UV_LEAPFROG, "jet")])
def test_hydrogen_thermodynamics_match_reference(scheme, state):
    """A hydrogen-helium atmosphere (x_h2 0.864, x_he 0.136: the reference's thermo_setup tables,
    return_temp and return_enthalpy by table interpolation) on the Held-Suarez planet: the
    restatement against the reference's step, every field bit for bit after every step."""
    if not reference_available():
        pytest.skip("reference source tree not present on this host")
    cfg = HSConfig(ni=32, nj=16, nk=10, dt=300, uv_scheme=scheme, seed=8, state=state,
                   profile=EPIC_PROFILE_N2 if state == "jet" else 0, x_h2=0.864, x_he=0.136)
    ga, f = hs_setup(cfg)
    sched = [("sync", 0)] + [("step", 1)] * 6
    geo, snaps = run_reference(ga, f, sched)
    port = Port(ga)
    port.upload(f)
    for i, (what, n) in enumerate(sched):
        if what == "sync":
            port.timestep(EPIC_SYNC_DIAGS_ONLY)
        else:
            port.run(n)
        got = port.download()
        want = dict_to_fields(snaps[i], 32, 16, 10, scheme)
        for k in got.arrays:
            assert np.array_equal(got.arrays[k], want.arrays[k]), f"snapshot {i}: field {k} differs"


@pytest.mark.parametrize("scheme,state,gg,direction,h2", [(EPIC_UV_AB3, "jet", False, 1, 0.), (EPIC_UV_LEAPFROG, "hs", False, 1, 0.),
                                                          (EPIC_UV_AB3, "jet", True, 1, 0.), (EPIC_UV_AB3, "jet", False, 2, 0.),
                                                          (EPIC_UV_AB3, "jet", False, 3, 0.), (EPIC_UV_AB3, "jet", True, 1, 0.864)])
def test_turbulence_matches_reference(scheme, state, gg, direction, h2):
    """The Spalart-Allmaras DES closure (source_sink_turb, the horizontal and vertical subgrid
    diffusion of THETA, NU_TURB and the winds, set_diffusion_coef in store_diag) on the
    Held-Suarez planet, terrestrial or gas-giant, ideal or hydrogen-helium: the restatement against the reference's step,
    every field (NU_TURB and the diffusivities included) bit for bit after every step."""
    if not reference_available():
        pytest.skip("reference source tree not present on this host")
    cfg = HSConfig(ni=32, nj=16, nk=10, dt=300, uv_scheme=scheme, seed=9, state=state,
                   profile=EPIC_PROFILE_N2 if state == "jet" else 0, gas_giant=gg, turbulence=True,
                   diffusion_direction=direction, x_h2=h2, x_he=0.136 if h2 else 0.)
    ga, f = hs_setup(cfg)
    sched = [("sync", 0)] + [("step", 1)] * 6
    geo, snaps = run_reference(ga, f, sched)
    port = Port(ga)
    port.upload(f)
    for i, (what, n) in enumerate(sched):
        if what == "sync":
            port.timestep(EPIC_SYNC_DIAGS_ONLY)
        else:
            port.run(n)
        got = port.download()
        want = dict_to_fields(snaps[i], 32, 16, 10, scheme)
        for k in got.arrays:
            assert np.array_equal(got.arrays[k], want.arrays[k]), f"snapshot {i}: field {k} differs"


@pytest.mark.parametrize("state,scheme", [("hs", EPIC_UV_AB3), ("jet", EPIC_UV_AB3), ("jet", EPIC_UV_LEAPFROG)])
def test_cfl_dt_matches_reference(state, scheme):
    """cfl_dt (the time step var_write stores before a save) of the restatement against the
    reference's, after the synchronising call and after steps."""
    if not reference_available():
        pytest.skip("reference source tree not present on this host")
    cfg = HSConfig(ni=32, nj=16, nk=10, dt=300, uv_scheme=scheme, seed=21, state=state,
                   profile=EPIC_PROFILE_N2 if state == "jet" else 0)
    ga, f = hs_setup(cfg)
    sched = [("sync", 0), ("step", 1), ("step", 3)]
    geo, snaps = run_reference(ga, f, sched)
    port = Port(ga)
    port.upload(f)
    for i, (what, n) in enumerate(sched):
        if what == "sync":
            port.timestep(EPIC_SYNC_DIAGS_ONLY)
        else:
            port.run(n)
        assert port.cfl_dt()[0] == snaps[i]["cfl_dt"], (i, port.cfl_dt(), snaps[i]["cfl_dt"])


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_libm_rounding_floor_at_64x32x10(seed):
    """The CUDA kernels equal the restatement with correctly rounded log/exp/pow bit for bit (the
    GPU tests check that); here that restatement stays within the drop-in bar of the glibc one,
    which reproduces the reference build, on the 64x32x10 Held-Suarez case after one step."""
    cfg = HSConfig(ni=64, nj=32, nk=10, dt=300, seed=seed)
    ga, f = hs_setup(cfg)
    out = []
    for cr in (False, True):
        p = Port(ga, cr_libm=cr)
        p.upload(f)
        p.timestep(EPIC_SYNC_DIAGS_ONLY)
        p.run(1)
        out.append(p.download())
    errs = field_errors(out[1], out[0], PROGNOSTIC)
    assert all(v[0] <= 1e-11 for v in errs.values()), errs


def test_akima_fixture_differs_from_hsu():
    """The Akima fixture's first step is not what the Hsu scheme gives from the same inputs, so
    the fixture (and every parity test that sets advection_scheme) exercises the Akima path."""
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "hs32x16x10_ab3_akima.npz"))
    ga = grid_from_fixture(z)
    assert ga.struct.advection_scheme == EPIC_ADV_AKIMA
    ga.struct.advection_scheme = EPIC_ADV_HSU
    port = Port(ga)
    port.upload(inputs_from_fixture(z, ga))
    port.timestep(EPIC_SYNC_DIAGS_ONLY)
    port.run(1)
    got = port.download()
    for k in ("hdry", "theta"):
        assert not np.array_equal(got.arrays[k], z["step1_" + k]), k


def test_jet_fixture_inputs_match_generator():
    """The jet fixture's inputs (constant-N^2 sounding grid, balanced jets, perturbation) equal
    what epic_hs_grid_build/epic_jet_initial_state produce now, and the state is a jet state:
    bottom pressure varying with latitude, zonal winds of tens of m/s."""
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "jet32x16x10_ab3.npz"))   # seed 15
    cfg = HSConfig(ni=32, nj=16, nk=10, dt=300, seed=15, profile=EPIC_PROFILE_N2, state="jet")
    ga, f = hs_setup(cfg)
    ga0 = grid_from_fixture(z)
    for k in ga.arrays:
        np.testing.assert_allclose(ga.arrays[k], ga0.arrays[k], rtol=1e-14, atol=0, err_msg=k)
    for k in ("p3", "theta", "hdry", "u", "v"):
        np.testing.assert_allclose(f.arrays[k], z["in_" + k], rtol=1e-12, atol=1e-12, err_msg=k)
    pbot = f.arrays["p3"][10, 1:18, 5]
    assert pbot.max() - pbot.min() > 5e3
    assert np.abs(f.arrays["u"][0][1:11]).max() > 50.


SOUNDING = os.path.join(os.path.dirname(__file__), "golden", "sounding", "t_vs_p_held_suarez.npz")


@pytest.mark.parametrize("shape", [(64, 32, 10), (512, 256, 40)])
def test_table_sounding_matches_reference_get_sounding(shape):
    """The grid build's theta profile from the reference's own Held-Suarez sounding (profile
    EPIC_PROFILE_TABLE) against the reference's get_sounding on the same table, at the grid's
    reference pressures: bit for bit."""
    from epic_gb300 import EPIC_PROFILE_TABLE
    from oracle_lib import reference_sounding_theta
    if not reference_available():
        pytest.skip("needs the reference source tree")
    z = np.load(SOUNDING)
    ni, nj, nk = shape
    ga, _ = hs_setup(HSConfig(ni=ni, nj=nj, nk=nk, dt=150, profile=EPIC_PROFILE_TABLE, table=(z["p"], z["t"])))
    kk = np.arange(2, 2 * nk + 1)
    want = reference_sounding_theta(z["p"], z["t"], ga.struct.press0, ga.p_ref[kk])
    got = ga.theta_ref[kk]
    assert np.array_equal(got, want), np.max(np.abs(got - want) / want)


def test_table_sounding_state():
    """The Held-Suarez state on the reference's sounding: sigmatheta decreasing downward, P3
    increasing downward in every column, theta of the pure-sigma layers near the table's."""
    from epic_gb300 import EPIC_PROFILE_TABLE
    z = np.load(SOUNDING)
    ga, f = hs_setup(HSConfig(ni=64, nj=32, nk=10, dt=300, profile=EPIC_PROFILE_TABLE, table=(z["p"], z["t"])))
    s = ga.struct
    sg = ga.sigmatheta[1:2 * s.nk + 2]
    assert np.all(np.diff(sg) < 0)
    p3 = f.p3[:s.nk + 1, 1:s.nj + 2, 1:s.ni + 1]
    assert np.all(np.diff(p3, axis=0) > 0)
    # the surface layer's theta follows the table's 1000 hPa temperature (288.15 K at 1013 hPa)
    th = f.theta[s.nk, 1:s.nj + 2, 1:s.ni + 1]
    assert 280. < th.mean() < 295.
