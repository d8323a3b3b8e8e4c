"""The drop-in step (epic_dropin_*, what the timestep() wrapper epic_gb300/dropin/epic_timestep_gb300.c
calls) driven the way the reference's driver loop drives timestep(): one SYNC_DIAGS_ONLY call to
prime, then per step timestep(STEP_PROGS_AND_SYNC_DIAGS) followed by grid.itime++ on the host
(src/shared/epic_main.c:303, :336-427), against the reference build's outputs stored in
tests/golden/*.npz.  Same bar as test_gpu_golden: relative L2 <= 1e-11 per field and step, or bit
equality with the correctly rounded restatement where that restatement is itself farther from the
reference than the bar (glibc's rounding of pow)."""
import ctypes as C
import glob
import os

import numpy as np
import pytest

from epic_gb300 import EPIC_PREC_FP64, EPIC_STEP_PROGS_AND_SYNC_DIAGS, EPIC_SYNC_DIAGS_ONLY, EpicError, load_library
from epic_gb300.abi import EpicFields, EpicGrid, Fields
from oracle_lib import Port
from test_gpu_golden import tolerance
from test_oracle import compare_snapshot, grid_from_fixture, inputs_from_fixture, snapshots

pytestmark = pytest.mark.gpu
GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))
MIRROR, RESIDENT = 0, 1   # EPIC_DROPIN_MIRROR, EPIC_DROPIN_RESIDENT


def _lib():
    lib = load_library()
    lib.epic_dropin_timestep.argtypes = [C.POINTER(EpicGrid), C.POINTER(EpicFields), C.c_int32, C.c_int32, C.c_int32,
                                         C.c_int64]
    lib.epic_dropin_sync_to_host.argtypes = [C.POINTER(EpicFields)]
    lib.epic_dropin_message.restype = C.c_char_p
    lib.epic_dropin_release.restype = None
    return lib


class Driver:
    """The reference driver loop's side of the contract: it owns grid.itime and the host `var`."""

    def __init__(self, ga, f, mode):
        self.lib, self.ga, self.f, self.mode, self.itime = _lib(), ga, f, mode, int(f.struct.itime)
        self.lib.epic_dropin_release()

    def timestep(self, action):
        rc = self.lib.epic_dropin_timestep(C.byref(self.ga.struct), C.byref(self.f.struct), EPIC_PREC_FP64, self.mode,
                                           action, self.itime)
        if rc:
            raise EpicError(self.lib.epic_dropin_message().decode())

    def prime(self):
        self.timestep(EPIC_SYNC_DIAGS_ONLY)

    def steps(self, n):
        for _ in range(n):
            self.timestep(EPIC_STEP_PROGS_AND_SYNC_DIAGS)
            self.itime += 1          # grid.itime++ after the call, epic_main.c:424

    def host_var(self):
        """What var_write would read: in resident mode the driver syncs first."""
        if self.mode == RESIDENT:
            rc = self.lib.epic_dropin_sync_to_host(C.byref(self.f.struct))
            assert rc == 0, self.lib.epic_dropin_message()
        return self.f

    def close(self):
        self.lib.epic_dropin_release()


@pytest.mark.parametrize("mode", [MIRROR, RESIDENT], ids=["mirror", "resident"])
@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def test_dropin_reference_loop(gpu, path, mode):
    z = np.load(path)
    ga = grid_from_fixture(z)
    f = inputs_from_fixture(z, ga)
    cr = Port(ga, cr_libm=True)
    cr.upload(f)
    d = Driver(ga, f.copy(), mode)
    done = 0
    try:
        for tag in snapshots(z):
            if tag == "sync":
                d.prime()
                cr.timestep(EPIC_SYNC_DIAGS_ONLY)
            else:
                n = int(tag[4:])
                d.steps(n - done)
                cr.run(n - done)
                done = n
            got = d.host_var()
            bad = compare_snapshot(got, z, tag, tolerance(tag))
            if bad:
                want = cr.download()
                floor = compare_snapshot(want, z, tag, tolerance(tag))
                assert set(bad) <= set(floor), (tag, bad)
                for k in bad:
                    assert np.array_equal(got.arrays[k], want.arrays[k]), (tag, k)
        assert d.lib.epic_dropin_status() == 0
    finally:
        d.close()


def test_dropin_keeps_the_first_error(gpu):
    """A state the reference stops on (negative potential temperature in one cell: GZ3 not
    monotonic) makes the first call fail with the reference's message; later calls return the
    same error without stepping, and the status reports it until the model is released."""
    from epic_gb300 import HSConfig, hs_setup
    ga, f = hs_setup(HSConfig(ni=32, nj=16, nk=10, dt=300, seed=91))
    f.theta[10, 5, 5] = -1.0
    d = Driver(ga, f, MIRROR)
    try:
        with pytest.raises(EpicError, match="GZ3 not monotonic"):
            d.prime()
        with pytest.raises(EpicError, match="GZ3 not monotonic"):
            d.steps(1)
        assert d.lib.epic_dropin_status() == -4    # EPIC_ERR_MODEL
    finally:
        d.close()
    assert d.lib.epic_dropin_status() == 0
