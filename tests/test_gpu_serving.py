"""The serving loop (epic_gb300/serving.py): runs of different shapes admitted by an HBM budget
and advanced in per-shape-class batches give each run the bits it gets alone."""
import numpy as np
import pytest

from epic_gb300 import EPIC_PREC_MIXED, HSConfig, hs_setup, model_bytes
from epic_gb300.serving import RunRequest, RunServer, latency_summary

pytestmark = pytest.mark.gpu


def _requests():
    shapes = [(32, 16, 10), (64, 32, 10), (32, 16, 10), (64, 32, 20), (32, 16, 10), (64, 32, 10)]
    steps = [9, 20, 33, 12, 17, 5]
    return [RunRequest(q, HSConfig(ni=a, nj=b, nk=c, dt=300, seed=50 + q), steps[q], arrival=0.002 * q,
                       kf_scale=1.0 + 0.03 * (q - 2)) for q, (a, b, c) in enumerate(shapes)]


def test_serving_results_equal_alone(gpu):
    reqs = _requests()
    # a budget that holds about three of these runs at a time, so admission has to wait
    need = [model_bytes(hs_setup(r.cfg)[0], EPIC_PREC_MIXED) for r in reqs]
    budget = sum(sorted(need)[-3:])
    mix = RunServer(hbm_budget=budget, precision=EPIC_PREC_MIXED, round_steps=4, keep_fields=True).serve(reqs)
    assert [r.rid for r in mix] == list(range(len(reqs)))
    for r, q in zip(mix, reqs):
        alone = RunServer(hbm_budget=budget, precision=EPIC_PREC_MIXED, round_steps=64, keep_fields=True).serve(
            [RunRequest(q.rid, q.cfg, q.steps, 0.0, q.kf_scale)])[0]
        for k in r.fields.arrays:
            assert np.array_equal(r.fields.arrays[k], alone.fields.arrays[k]), (q.rid, k)
        assert r.fields.struct.itime == q.steps
    s = latency_summary(mix)
    assert s["p99_s"] >= s["p50_s"] > 0 and s["aggregate_cell_steps_per_s"] > 0


def test_serving_rejects_oversized_request(gpu):
    q = RunRequest(0, HSConfig(ni=64, nj=32, nk=10, dt=300), 3)
    with pytest.raises(ValueError, match="budget"):
        RunServer(hbm_budget=1 << 20).serve([q])
