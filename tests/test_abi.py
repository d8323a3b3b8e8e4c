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
