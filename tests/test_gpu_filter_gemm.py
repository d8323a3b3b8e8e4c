"""The zonal filter of whole planes on the tensor cores (k_filter_planes_gemm, the mixed form's
path for ni a multiple of 128) against the FP64 form's FFT filter: the diagnostics that
store_diag filters (PV3 from the filtered V, DIV_UV3 from the filtered U and V) after one call
of the stage on the same state, for one (ni = 128), two (ni = 256) and four (ni = 512) 128-point
output tiles per row.  3xTF32 products keep FP32 accuracy, so the two agree to FP32 level (measured on a GB300:
PV3 ~8e-8, DIV_UV3 ~4e-7 relative L2); the bounds leave a factor ~10."""
import pytest

from compare import field_errors
from epic_gb300 import EPIC_PREC_FP64, EPIC_PREC_MIXED, EPIC_SYNC_DIAGS_ONLY, HSConfig, Model, hs_setup

pytestmark = pytest.mark.gpu
STORE_DIAG = 16


@pytest.mark.parametrize("shape,dt", [((128, 64, 10), 150), ((256, 128, 10), 120), ((512, 256, 10), 60)])
def test_tensor_core_filter_matches_fp64(gpu, shape, dt):
    ni, nj, nk = shape
    ga, f = hs_setup(HSConfig(ni=ni, nj=nj, nk=nk, dt=dt, seed=5))
    spin = Model(ga, EPIC_PREC_FP64)
    spin.upload(f)
    spin.timestep(EPIC_SYNC_DIAGS_ONLY)
    spin.run(4)
    spin.sync()
    state = spin.download()
    out = {}
    for prec in (EPIC_PREC_FP64, EPIC_PREC_MIXED):
        m = Model(ga, prec)
        m.upload(state)
        m.run_stage(STORE_DIAG)
        m.sync()
        out[prec] = m.download()
    e = field_errors(out[EPIC_PREC_MIXED], out[EPIC_PREC_FP64], ["pv3", "div_uv3"])
    assert e["pv3"][0] < 1e-6 and e["div_uv3"][0] < 5e-6, e
