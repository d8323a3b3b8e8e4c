"""epic_model_filter_mass_noalloc (the 3-D mass filter with its profile tables in the library's
fixed device array) against epic_model_run_stage(m, 10) (the same filter with the model's own
scratch), two calls in a row on the same spun-up state.  Collected last so that it also runs
after every other GPU test in the same process."""
import numpy as np
import pytest

from epic_gb300 import EPIC_PREC_FP64, EPIC_PREC_MIXED, EPIC_SYNC_DIAGS_ONLY, EpicError, HSConfig, Model, hs_setup
from oracle_lib import Port

pytestmark = pytest.mark.gpu

NOALLOC_TABLE_ENTRIES = 16384   # EPIC_NOALLOC_TABLE_ENTRIES in include/epic_gb300.h


def _spun_up(cfg, nsteps):
    ga, f = hs_setup(cfg)
    port = Port(ga)
    port.upload(f)
    port.timestep(EPIC_SYNC_DIAGS_ONLY)
    port.run(nsteps)
    return ga, port.download()


@pytest.mark.parametrize("shape,precision", [((32, 16, 10), EPIC_PREC_FP64), ((64, 32, 20), EPIC_PREC_FP64),
                                              ((32, 16, 10), EPIC_PREC_MIXED), ((128, 64, 20), EPIC_PREC_MIXED)])
def test_noalloc_filter_matches_stage(gpu, shape, precision):
    """Both precision forms: the mixed form's filter has its own shared-memory layout (profile
    intervals, FP32 row) and filters only the filtered rows; at ni = 128 its filtered GZ copy
    (stage 8) runs on the tensor cores."""
    ni, nj, nk = shape
    ga, f = _spun_up(HSConfig(ni=ni, nj=nj, nk=nk, dt=300, seed=7), 3)
    ref, fixed = Model(ga, precision), Model(ga, precision)
    for m in (ref, fixed):
        m.upload(f)
        m.run_stage(8)   # the filtered GZ copy whose bottom row and profiles the 3-D filter reads
    for call in range(2):
        ref.run_stage(10)
        fixed.filter_mass_noalloc()
        ref.sync()
        fixed.sync()
        a, b = ref.download(), fixed.download()
        for k in a.arrays:
            assert np.array_equal(a.arrays[k], b.arrays[k]), f"call {call + 1}: field {k} differs"
    # the filter did something: HDRY differs from the input in the filtered rows
    assert not np.array_equal(a.arrays["hdry"], f.arrays["hdry"])


def test_noalloc_filter_rejects_grids_beyond_its_table(gpu):
    ni, nj, nk = 4, 200, 100
    assert (nj + 3) * (nk + 2) > NOALLOC_TABLE_ENTRIES
    ga, _ = hs_setup(HSConfig(ni=ni, nj=nj, nk=nk, dt=300))
    m = Model(ga)
    with pytest.raises(EpicError, match="exceeds"):
        m.filter_mass_noalloc()
