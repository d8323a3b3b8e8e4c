"""Asynchronous snapshots (epic_model_snapshot_begin/_wait): the state copied out at one step
while the model keeps stepping equals the state of a model stopped there, and taking it does not
disturb the run."""
import numpy as np
import pytest

from epic_gb300 import EPIC_PREC_FP64, EPIC_PREC_MIXED, EPIC_SYNC_DIAGS_ONLY, Fields, HSConfig, Model, hs_setup

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [EPIC_PREC_FP64, EPIC_PREC_MIXED])
def test_snapshot_while_stepping(gpu, precision):
    ga, f = hs_setup(HSConfig(ni=64, nj=32, nk=10, dt=300, seed=21))

    def fresh():
        m = Model(ga, precision)
        m.upload(f)
        m.timestep(EPIC_SYNC_DIAGS_ONLY)
        return m

    a = fresh()
    a.run(5)
    snap = Fields(64, 32, 10, ga.struct.uv_scheme, pinned=True)
    a.snapshot_begin(snap)
    a.run(7)                      # enqueued behind the device-side copy; overlaps the host copy
    got = a.snapshot_wait()
    a.sync()
    b = fresh()
    b.run(5)
    b.sync()
    want = b.download()
    for k in want.arrays:
        assert np.array_equal(got.arrays[k], want.arrays[k]), k
    assert (got.struct.itime, got.struct.it_zero) == (want.struct.itime, want.struct.it_zero)
    c = fresh()
    c.run(12)
    c.sync()
    x, y = a.download(), c.download()
    for k in x.arrays:
        assert np.array_equal(x.arrays[k], y.arrays[k]), k
