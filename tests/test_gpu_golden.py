"""The CUDA step, from the inputs stored in tests/golden/*.npz, against the reference build's
outputs stored there (made by tests/golden/make_golden.py from the reference sources).

Bar: relative L2 <= 1e-11 per field after the synchronising call and after the first step,
1e-11 per step taken after that.  The kernels evaluate log/exp/pow correctly rounded; glibc's
pow, which the reference calls, is not in about 0.1% of calls, and a one-ulp difference in P2
or T3 moves U by ~1e-11 after one step from rest.  Where the restatement with correctly rounded
functions (oracle libepicport_cr.so) is itself farther than the bar from the reference, the
GPU result must equal that restatement bit for bit instead (the gap is then glibc's rounding,
not the kernels')."""
import glob
import os

import numpy as np
import pytest

from epic_gb300 import EPIC_SYNC_DIAGS_ONLY, Model
from oracle_lib import Port
from test_oracle import compare_snapshot, grid_from_fixture, inputs_from_fixture, snapshots

pytestmark = pytest.mark.gpu
GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))


def tolerance(tag):
    return 1e-11 if tag in ("sync", "step1") else 1e-11 * int(tag[4:])


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def test_golden_gpu(gpu, path):
    z = np.load(path)
    ga = grid_from_fixture(z)
    f = inputs_from_fixture(z, ga)
    m = Model(ga)
    m.upload(f)
    cr = Port(ga, cr_libm=True)
    cr.upload(f)
    done = 0
    for tag in snapshots(z):
        if tag == "sync":
            m.timestep(EPIC_SYNC_DIAGS_ONLY)
            cr.timestep(EPIC_SYNC_DIAGS_ONLY)
        else:
            n = int(tag[4:])
            m.run(n - done)
            cr.run(n - done)
            done = n
        m.sync()
        got = m.download()
        bad = compare_snapshot(got, z, tag, tolerance(tag))
        if bad:
            want = cr.download()
            floor = compare_snapshot(want, z, tag, tolerance(tag))
            assert set(bad) <= set(floor), (tag, bad, "the correctly rounded restatement meets the bar here")
            for k in bad:
                assert np.array_equal(got.arrays[k], want.arrays[k]), (tag, k, bad[k], floor[k])
