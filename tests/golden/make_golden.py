"""Generate the golden fixtures in this directory from the reference build (run where the
reference source tree is available; the fixtures travel, the reference does not).

Each fixture holds the inputs (grid scalars and arrays, the initial state) and the reference's
state after timestep(SYNC_DIAGS_ONLY) and after a number of timestep(STEP_PROGS_AND_SYNC_DIAGS)
calls, computed by oracle/_ref/libepicref.so (the reference's own sources, driven in-process).

    python tests/golden/make_golden.py [case ...]     (all cases when none is named)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from epic_gb300 import EPIC_ADV_AKIMA, EPIC_PROFILE_N2, EPIC_UV_AB3, EPIC_UV_LEAPFROG, HSConfig, hs_setup  # noqa: E402
from oracle_lib import reference_available, run_reference, fields_to_dict  # noqa: E402

SAVED = ("u", "v", "hdry", "theta", "p3", "gz3", "pv3", "w3", "heat3", "div_uv3", "gz_surface")
CASES = {
    "hs32x16x10_ab3": (HSConfig(ni=32, nj=16, nk=10, dt=300, uv_scheme=EPIC_UV_AB3, seed=11), [("sync", 0), ("step", 1), ("step", 4)]),
    "hs32x16x10_leapfrog": (HSConfig(ni=32, nj=16, nk=10, dt=300, uv_scheme=EPIC_UV_LEAPFROG, seed=12), [("sync", 0), ("step", 1), ("step", 2)]),
    "hs16x8x12_ab3": (HSConfig(ni=16, nj=8, nk=12, dt=600, uv_scheme=EPIC_UV_AB3, seed=13), [("sync", 0), ("step", 3)]),
    "hs32x16x10_ab3_akima": (HSConfig(ni=32, nj=16, nk=10, dt=300, uv_scheme=EPIC_UV_AB3, seed=14, advection_scheme=EPIC_ADV_AKIMA),
                             [("sync", 0), ("step", 1), ("step", 4)]),
    "jet32x16x10_ab3": (HSConfig(ni=32, nj=16, nk=10, dt=300, uv_scheme=EPIC_UV_AB3, seed=15, profile=EPIC_PROFILE_N2, state="jet"),
                        [("sync", 0), ("step", 1), ("step", 4)]),
    # the jets over the gas-giant lower boundary (planet->type "gas-giant": GZ_SURFACE from gz_from_u)
    "jetgg32x16x10_ab3": (HSConfig(ni=32, nj=16, nk=10, dt=300, uv_scheme=EPIC_UV_AB3, seed=16, profile=EPIC_PROFILE_N2, state="jet",
                                   gas_giant=True), [("sync", 0), ("step", 1), ("step", 4)]),
    # the jets with the Spalart-Allmaras DES turbulence closure (grid.turbulence_scheme on)
    "jetsa32x16x10_ab3": (HSConfig(ni=32, nj=16, nk=10, dt=300, uv_scheme=EPIC_UV_AB3, seed=17, profile=EPIC_PROFILE_N2, state="jet",
                                   turbulence=True), [("sync", 0), ("step", 1), ("step", 4)]),
    # the column in a hydrogen-helium atmosphere (thermo_setup's tables, x_h2 = 0.864, x_he = 0.136)
    "hsh2_32x16x10_ab3": (HSConfig(ni=32, nj=16, nk=10, dt=300, uv_scheme=EPIC_UV_AB3, seed=18, x_h2=0.864, x_he=0.136),
                          [("sync", 0), ("step", 1), ("step", 4)]),
}


def make(name, cfg, schedule):
    ga, f = hs_setup(cfg)
    geo, snaps = run_reference(ga, f, schedule)
    out = {"geometry_maxdiff": np.array(geo)}
    for k, v in ga.arrays.items():
        out["grid_" + k] = v
    for k, v in ga.scalars().items():
        out["scalar_" + k] = np.array(v)
    d = fields_to_dict(f)
    for k in ("u", "v", "dudt", "dvdt", "hdry", "theta", "p3", "gz_surface", "u_spinup") + (("nu_turb",) if cfg.turbulence else ()):
        out["in_" + k] = d[k]
    for n in ("it_zero", "it_minus1", "it_minus2", "itime", "model_time"):
        out["in_" + n] = np.array(d[n])
    steps_done = 0
    for (what, n), s in zip(schedule, snaps):
        steps_done += n
        tag = "sync" if what == "sync" else f"step{steps_done}"
        for k in SAVED + (("nu_turb", "diffusion_coef_theta", "diffusion_coef_uv") if cfg.turbulence else ()):
            out[f"{tag}_{k}"] = s[k]
        for n2 in ("it_zero", "it_minus1", "it_minus2", "itime", "model_time"):
            out[f"{tag}_{n2}"] = np.array(s[n2])
    out["schedule"] = np.array([f"{w}:{n}" for w, n in schedule])
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    if not reference_available():
        sys.exit("the reference source tree is needed to generate the fixtures")
    for name in sys.argv[1:] or CASES:
        make(name, *CASES[name])
