"""The serving loop's scheduling (epic_gb300/serving.py) with a stand-in for the device: admission
by memory budget with backfill, one batch per shape class, exact step counts when runs join a
class whose batch is still running, and retirement returning memory to the budget.  No GPU is
needed."""
from types import SimpleNamespace

import numpy as np
import pytest

from epic_gb300 import HSConfig
from epic_gb300.serving import RunRequest, RunServer, latency_summary


class FakeModel:
    def __init__(self, cfg):
        self.cfg, self.steps, self.closed = cfg, 0, False

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
        pass

    def close(self):
        pass


class FakeBackend:
    """Device bytes = cells (so that the budget is easy to reason about)."""

    def __init__(self, lag=0):
        self.models, self.log, self.lag = [], [], lag

    def setup(self, cfg):
        return SimpleNamespace(struct=SimpleNamespace(hs_kf=1.0), cfg=cfg), None

    def bytes(self, grid, precision):
        c = grid.cfg
        return c.ni * c.nj * c.nk

    def model(self, grid, fields, precision):
        m = FakeModel(grid.cfg)
        self.models.append(m)
        return m

    def batch(self, models):
        return FakeBatch(self.log, models, self.lag)


def _req(rid, shape, steps, arrival=0.0):
    ni, nj, nk = shape
    return RunRequest(rid, HSConfig(ni=ni, nj=nj, nk=nk), steps, arrival=arrival)


@pytest.mark.parametrize("lag", [0, 3])
def test_budget_backfill_classes_and_step_counts(lag):
    be = FakeBackend(lag)
    big, small = (64, 32, 10), (16, 8, 10)          # 20480 and 1280 "bytes"
    reqs = [_req(0, big, 7), _req(1, big, 5), _req(2, small, 9), _req(3, small, 4), _req(4, big, 3)]
    server = RunServer(hbm_budget=20480 + 2 * 1280, round_steps=4, backend=be)
    res = server.serve(reqs)
    assert [r.rid for r in res] == [0, 1, 2, 3, 4]
    assert server.peak_used <= server.hbm_budget and server.used == 0
    # every run stepped exactly its count, and its model was released
    assert sorted(m.steps for m in be.models) == sorted(q.steps for q in reqs)
    assert all(m.closed for m in be.models)
    # a batch never mixes shapes; the two small runs were admitted beside the first big one
    assert all(len(shapes) == 1 for _, shapes, _ in be.log)
    assert any(n == 2 and shapes == {small} for n, shapes, _ in be.log)
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
