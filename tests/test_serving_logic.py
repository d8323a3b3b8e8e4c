"""The serving loop's scheduling (epic_gb300/serving.py) with a stand-in for the device: admission
by memory budget with backfill, one batch per shape class, exact step counts when runs join a
class whose batch is still running, and retirement returning memory to the budget.  No GPU is
needed."""
from types import SimpleNamespace

import numpy as np
import pytest

from epic_gb300 import HSConfig
from epic_gb300.abi import EPIC_DIFFUSION_JUST_VERTICAL
from epic_gb300.serving import RunRequest, RunServer, latency_summary


class FakeModel:
    def __init__(self, cfg, fail_at=None):
        self.cfg, self.steps, self.closed, self.fail_at = cfg, 0, False, fail_at

    @property
    def failed(self):
        return self.fail_at is not None and self.steps >= self.fail_at

    def download(self):
        a = np.full((2, 2), float(self.steps))
        return SimpleNamespace(arrays={"u": a, "v": a, "hdry": a, "theta": a})

    def close(self):
        self.closed = True


class FakeBatch:
    """Reports done only after `lag` polls, like a batch still busy on its stream."""

    def __init__(self, log, models, lag):
        self.log, self.models, self.lag, self.polls = log, list(models), lag, 0

    def run(self, n):
        shapes = {(m.cfg.ni, m.cfg.nj, m.cfg.nk) for m in self.models}
        self.log.append((len(self.models), shapes, n))
        for m in self.models:
            m.steps += n
        self.polls = 0

    def done(self):
        self.polls += 1
        return self.polls > self.lag

    def sync(self):
        from epic_gb300 import EpicError
        if any(m.failed for m in self.models):
            raise EpicError("member failed")

    def close(self):
        pass


class FakeBackend:
    """Device bytes = cells (so that the budget is easy to reason about)."""

    def __init__(self, lag=0, fail_at=None):
        self.models, self.log, self.lag = [], [], lag
        self.fail_at = fail_at or {}   # request seed -> step count at which its model errs

    def setup(self, cfg):
        return SimpleNamespace(struct=SimpleNamespace(hs_kf=1.0), cfg=cfg), None

    def bytes(self, grid, precision):
        c = grid.cfg
        return c.ni * c.nj * c.nk

    def model(self, grid, fields, precision):
        m = FakeModel(grid.cfg, self.fail_at.get(grid.cfg.seed))
        self.models.append(m)
        return m

    def batch(self, models):
        return FakeBatch(self.log, models, self.lag)

    def failures(self, models):
        return {q: "model error" for q, m in enumerate(models) if m.failed}


def _req(rid, shape, steps, arrival=0.0):
    ni, nj, nk = shape
    return RunRequest(rid, HSConfig(ni=ni, nj=nj, nk=nk, seed=rid), steps, arrival=arrival)


@pytest.mark.parametrize("lag", [0, 3])
def test_budget_backfill_classes_and_step_counts(lag):
    be = FakeBackend(lag)
    big, small = (64, 32, 10), (16, 8, 10)          # 20480 and 1280 "bytes"
    reqs = [_req(0, big, 7), _req(1, big, 5), _req(2, small, 9), _req(3, small, 4), _req(4, big, 3)]
    server = RunServer(hbm_budget=20480 + 2 * 1280, round_steps=4, backend=be, size_ratio=0)
    res = server.serve(reqs)
    assert [r.rid for r in res] == [0, 1, 2, 3, 4]
    assert server.peak_used <= server.hbm_budget and server.used == 0
    # every run stepped exactly its count, and its model was released
    assert sorted(m.steps for m in be.models) == sorted(q.steps for q in reqs)
    assert all(m.closed for m in be.models)
    # a batch never mixes layer counts (a launch class); the two small runs were admitted beside
    # the first big one and share its class, so they are batched with it
    assert all(len({nk for _, _, nk in shapes}) == 1 for _, shapes, _ in be.log)
    assert any(n == 3 and shapes == {small, big} for n, shapes, _ in be.log)
    assert all(n <= 4 for _, _, n in be.log)
    s = latency_summary(res)
    assert s["requests"] == 5 and s["p99_s"] >= s["p50_s"]


def test_run_joining_a_busy_class_steps_exactly_its_count():
    """A run admitted while its class's batch is still running joins the next batch and is not
    charged for the steps of the one in flight."""
    be = FakeBackend(lag=50)
    shape = (32, 16, 10)
    reqs = [_req(0, shape, 40), _req(1, shape, 6, arrival=0.002), _req(2, shape, 11, arrival=0.004)]
    server = RunServer(hbm_budget=10 * 32 * 16 * 10, round_steps=5, backend=be)
    res = server.serve(reqs)
    assert [r.rid for r in res] == [0, 1, 2]
    assert [m.steps for m in be.models] == [40, 6, 11]
    assert max(n for n, _, _ in be.log) >= 2          # the later runs did join run 0's batch


def test_oversized_request_is_rejected():
    with pytest.raises(ValueError, match="budget"):
        RunServer(hbm_budget=100, backend=FakeBackend()).serve([_req(0, (64, 32, 10), 2)])


def test_run_ended_by_a_model_error_is_retired_and_the_rest_go_on():
    """A run whose model reports an error (the device halts it) is retired with that error and its
    memory returns to the budget; the other run of its class and a later one still complete."""
    be = FakeBackend(fail_at={1: 5})
    shape = (32, 16, 10)
    reqs = [_req(0, shape, 12), _req(1, shape, 12), _req(2, shape, 8, arrival=0.003)]
    server = RunServer(hbm_budget=2 * 32 * 16 * 10, round_steps=4, backend=be)
    res = server.serve(reqs)
    assert [r.rid for r in res] == [0, 1, 2]
    assert res[1].error == "model error" and res[0].error is None and res[2].error is None
    assert [m.steps for m in be.models] == [12, 8, 8]
    assert server.used == 0 and all(m.closed for m in be.models)
    s = latency_summary(res)
    assert s["completed"] == 2 and s["ended_by_model_error"] == 1


def test_durations_in_simulated_days():
    from epic_gb300.serving import poisson_requests
    reqs = poisson_requests(30, 20.0, 5, [(64, 32, 10), (128, 64, 20)], dt_of=lambda s: 300, jet_frac=0.5,
                            jet_dt_of=lambda s: 60, days_range=(0.25, 2.0))
    assert any(r.cfg.state == "jet" for r in reqs) and any(r.cfg.state == "hs" for r in reqs)
    for r in reqs:
        days = r.steps * r.cfg.dt / 86400.0
        assert 0.25 - 1e-3 <= days <= 2.0 + 1e-3
    assert all(np.diff([r.arrival for r in reqs]) > 0)


def test_launch_class_separates_physics_a_batch_must_share():
    """Runs over the gas-giant boundary, with the hydrogen tables or with the turbulence closure
    (per diffusion direction) each form their own launch class (epic_batch_create refuses to mix
    them); the seed, drag scale and initial state do not split a class."""
    from epic_gb300.serving import launch_class
    base = HSConfig(ni=32, nj=16, nk=10)
    variants = [HSConfig(ni=32, nj=16, nk=10, gas_giant=True), HSConfig(ni=32, nj=16, nk=10, x_h2=0.864, x_he=0.136),
                HSConfig(ni=32, nj=16, nk=10, turbulence=True),
                HSConfig(ni=32, nj=16, nk=10, turbulence=True, diffusion_direction=EPIC_DIFFUSION_JUST_VERTICAL)]
    keys = [launch_class(c, 10, 0) for c in [base] + variants]
    assert len(set(keys)) == len(keys)
    assert launch_class(HSConfig(ni=32, nj=16, nk=10, seed=5, state="jet"), 10, 0) == keys[0]


def test_size_buckets_keep_small_runs_out_of_large_batches():
    """With size buckets (the default: powers of 16 in cells) a small run is not batched with a run
    64 times its size, but is with one 4 times its size; with size_ratio=0 all three share one."""
    from epic_gb300.serving import launch_class
    small, mid, big = HSConfig(ni=32, nj=16, nk=10), HSConfig(ni=64, nj=32, nk=10), HSConfig(ni=128, nj=64, nk=10)
    assert launch_class(small, 10, 0) != launch_class(big, 10, 0)      # FP64: one filter path
    assert launch_class(small, 10, 0) == launch_class(mid, 10, 0)
    assert launch_class(small, 10, 0, 0) == launch_class(big, 10, 0, 0)
    be = FakeBackend()
    reqs = [_req(0, (32, 16, 10), 6), _req(1, (256, 128, 10), 6), _req(2, (64, 32, 10), 6)]
    RunServer(hbm_budget=10 ** 9, round_steps=3, backend=be).serve(reqs)
    assert all(len(shapes) == 1 or shapes == {(32, 16, 10), (64, 32, 10)} for _, shapes, _ in be.log)
