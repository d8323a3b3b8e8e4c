"""The C ABI library: it loads, exports what include/*.h declares, and its host-only entry
points work without a GPU.  No kernel runs here."""
import ctypes as C
import glob
import os
import re

import numpy as np
import pytest

import epic_gb300
from epic_gb300 import EpicError, HSConfig, hs_setup

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:[A-Za-z_][\w\s\*]*?)\b([a-z_][a-z0-9_]*)\s*\(", text, flags=re.M):
            if m.group(1) not in ("if", "sizeof", "return"):
                names.add(m.group(1))
    return sorted(names)


def test_library_exports_every_declared_symbol(cuda_lib):
    names = declared_functions()
    assert "epic_model_timestep" in names and len(names) >= 14
    missing = [n for n in names if not hasattr(cuda_lib, n)]
    assert not missing, missing


def test_grid_build_held_suarez(cuda_lib):
    ga, f = hs_setup(HSConfig(ni=64, nj=32, nk=10, dt=300))
    s = ga.struct
    assert s.k_sigma == 10 and 0 < s.sigma_sigma < 1
    sg = ga.sigmatheta[1:2 * s.nk + 2]
    assert np.all(np.diff(sg) < 0), "sigmatheta must decrease downward"
    assert np.all(ga.h_min[1:s.nk + 1] > 0)
    assert ga.lat[0] == -90. and ga.lat[-1] == 90.
    np.testing.assert_allclose(ga.lat, -ga.lat[::-1], rtol=0, atol=1e-12)
    # the state is at rest and hydrostatic-ready: P3 increases downward in every column
    p3 = f.p3[:s.nk + 1, 1:s.nj + 2, 1:s.ni + 1]
    assert np.all(np.diff(p3, axis=0) > 0)
    assert np.all(f.u == 0) and np.all(f.v == 0)
    # AB3 start flags in the two older tendency planes
    assert np.all(f.dudt[1][1:s.nk + 1, 1:s.nj + 2, 1:s.ni + 1] == np.finfo(float).max)


def test_seeded_noise_is_reproducible_and_seed_dependent(cuda_lib):
    a = hs_setup(HSConfig(ni=32, nj=16, nk=10, seed=1))[1].theta
    b = hs_setup(HSConfig(ni=32, nj=16, nk=10, seed=1))[1].theta
    c = hs_setup(HSConfig(ni=32, nj=16, nk=10, seed=2))[1].theta
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    noise = (a - c)[9:11, 1:18, 1:33]
    assert 0.05 < np.std(noise) / np.sqrt(2) < 0.2


def test_bad_arguments_are_errors_not_exits(cuda_lib):
    with pytest.raises(EpicError, match="power of 2"):
        hs_setup(HSConfig(ni=60, nj=32, nk=10))
    lib = cuda_lib
    rc = lib.epic_model_timestep(None, 0)
    assert rc == -1
    assert b"NULL" in lib.epic_last_error()


def test_model_needs_a_gpu_here():
    """Without a CUDA device the step fails loudly instead of falling back to the CPU."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    ga, _ = hs_setup(HSConfig(ni=16, nj=8, nk=6))
    with pytest.raises(EpicError):
        epic_gb300.Model(ga)


def test_dropin_wrapper_links_in_place_of_the_reference_step(cuda_lib):
    """epic_gb300/dropin/epic_timestep_gb300.c, compiled with the reference's headers, linked with
    the reference's objects in place of its timestep() (oracle/Makefile `dropin`) and driven by the
    reference harness: its timestep() is the one reached, and without a GPU it ends the run the
    reference's way, epic_error() naming timestep and the CUDA failure, exit status 1."""
    import subprocess
    import sys
    from oracle_lib import ORACLE, REF_ARGS, reference_available
    if not reference_available():
        pytest.skip("needs the reference source tree")
    r = subprocess.run(["make", "-s", "-C", ORACLE, "dropin", *REF_ARGS], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present: tests/test_gpu_dropin.py covers the step")
    code = (
        "import ctypes as C, sys\n"
        f"sys.path[:0] = [{ROOT!r}, {os.path.join(ROOT, 'tests')!r}]\n"
        "from epic_gb300 import HSConfig, hs_setup\n"
        "ga, f = hs_setup(HSConfig(ni=32, nj=16, nk=10, dt=300))\n"
        f"lib = C.CDLL({os.path.join(ORACLE, '_ref', 'libepicref_dropin.so')!r})\n"
        "assert lib.ref_init(C.byref(ga.struct), C.byref(f.struct)) == 0\n"
        "lib.ref_timestep(1)\n"
        "print('returned')\n")
    p = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    out = p.stdout + p.stderr
    assert p.returncode == 1 and "returned" not in out, out
    assert "EPIC Error" in out and "timestep" in out, out
