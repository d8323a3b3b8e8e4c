"""Serving: a request loop that keeps many runs of different shapes on one GPU.

The reference runs one model per process and has no serving layer; this module is new.  A
request is one synthetic Held-Suarez run (shape, time step, seed, drag-rate scale, number of
steps).  The server

  * admits waiting requests, in arrival order with backfill, while the device bytes of the
    admitted runs (epic_model_bytes) stay within its HBM budget;
  * keeps every admitted run's state on the device from admission to completion;
  * groups the active runs by launch class -- what the runs of one Batch must share: layers,
    schemes, precision form, viscosity orders, and in the mixed forms the zonal filter's path;
    grid sizes and time steps may differ, within a size bucket (a power of 16 in cells by
    default, since a batch steps at its largest member's pace) -- and advances each class as one
    Batch: every kernel of a step is launched once for all of the class's runs, uneven sizes
    included, and the classes' batches run on their own streams, so their work overlaps on the
    device;
  * never waits on one class while another could be launched: each pass polls every class's
    batch (epic_batch_query), settles the ones that finished and relaunches them at once;
  * re-forms a class's batch whenever a run joins or leaves it (continuous batching: runs that
    arrive while others are on the GPU join when their class's batch in flight finishes);
  * retires a run when its steps are done: its state is copied to the host and its device
    memory returns to the budget;
  * retires a run whose step recorded a fatal model error (where the reference's epic_error()
    would end the run) with that error: the model halts on the device, its memory returns to the
    budget, and the other runs of its class go on.

Each run's result is the same bits it gets when run alone (a batch gives every member the bits
of its own step, and the number of steps per round does not change the arithmetic).
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field

import numpy as np

from . import (Batch, EPIC_PREC_FP64, EPIC_PREC_MIXED, EPIC_PROFILE_N2, EPIC_SYNC_DIAGS_ONLY, EpicError, Fields, HSConfig, Model, hs_setup,
               model_bytes)


@dataclass
class RunRequest:
    rid: int
    cfg: HSConfig
    steps: int
    arrival: float = 0.0          # seconds after the server starts
    kf_scale: float = 1.0         # Held-Suarez drag rate k_f multiplier


@dataclass
class RunResult:
    rid: int
    shape: tuple
    steps: int
    arrival: float
    admitted: float
    finished: float
    fields: Fields | None = None
    checksum: float = 0.0
    error: str | None = None      # the model error that ended the run early, if any

    @property
    def latency(self) -> float:
        return self.finished - self.arrival


@dataclass
class _Active:
    req: RunRequest
    model: Model
    bytes: int
    remaining: int
    admitted: float


def launch_class(cfg: HSConfig, k_sigma: int, precision: int, size_ratio: int = 16) -> tuple:
    """What the members of one Batch must share (epic_batch_create): layers and the pure-sigma
    split, schemes, precision form, which viscosity orders and whether divergence damping act,
    the filter latitude, the lower boundary (gas giant or terrain), the thermodynamics (hydrogen
    tables or the ideal gas), the turbulence closure and its diffusion directions, and in the
    mixed forms whether ni takes the tensor-core filter -- plus a
    size bucket: a batch's step takes as long as its largest member's, so runs are batched only
    with runs whose cell count lies in the same power of size_ratio (0 batches every size of a
    class together)."""
    tensor_filter = precision != EPIC_PREC_FP64 and cfg.ni % 128 == 0 and cfg.ni <= 1024
    bucket = int(math.log(cfg.ni * cfg.nj * cfg.nk, size_ratio)) if size_ratio > 1 else 0
    return (cfg.nk, k_sigma, cfg.uv_scheme, cfg.advection_scheme, precision, tensor_filter, cfg.nu4 > 0, cfg.nu6 > 0,
            cfg.nu8 > 0, cfg.nudiv != 0, cfg.lat0, cfg.gas_giant, cfg.x_h2 > 0,
            cfg.diffusion_direction if cfg.turbulence else None, bucket)


def state_checksum(f: Fields) -> float:
    """Sum of |U| + |V| + |HDRY| + |THETA| over the current planes (a compact result summary)."""
    tot = 0.0
    for k in ("u", "v", "hdry", "theta"):
        a = f.arrays[k]
        tot += float(np.abs(np.where(np.abs(a) > 1e300, 0., a)).sum())
    return tot


class DeviceBackend:
    """What the server needs from the library (the CPU tests of the scheduling logic replace it)."""

    def setup(self, cfg: HSConfig):
        return hs_setup(cfg)

    def bytes(self, grid, precision: int) -> int:
        return model_bytes(grid, precision)

    def model(self, grid, fields, precision: int):
        m = Model(grid, precision)
        m.upload(fields)
        m.timestep(EPIC_SYNC_DIAGS_ONLY)
        return m

    def batch(self, models):
        return Batch(models)

    def failures(self, models) -> dict:
        """Index -> message of every model whose device-side error record is set."""
        out = {}
        for q, m in enumerate(models):
            try:
                m.sync()
            except EpicError as e:
                out[q] = str(e)
        return out


@dataclass
class RunServer:
    hbm_budget: int                      # bytes of device memory the admitted runs may hold
    precision: int = EPIC_PREC_MIXED
    round_steps: int = 16                # most steps a class advances per scheduling pass
    keep_fields: bool = False            # keep each result's full state (else a checksum)
    size_ratio: int = 16                 # runs share a batch only in one power of this in cells (0: any)
    allow_jets: bool = True              # serve jet-state requests (a server may refuse them)
    backend: object = field(default_factory=DeviceBackend)
    waiting: list = field(default_factory=list)
    prepared: dict = field(default_factory=dict)    # rid -> (grid, initial fields, device bytes)
    active: dict = field(default_factory=dict)      # launch class -> list[_Active]
    batches: dict = field(default_factory=dict)     # launch class -> (Batch, member ids)
    inflight: dict = field(default_factory=dict)    # launch class -> (Batch, steps, members) running
    results: list = field(default_factory=list)
    used: int = 0
    peak_used: int = 0
    t0: float = 0.0

    def now(self) -> float:
        return time.perf_counter() - self.t0

    def submit(self, req: RunRequest) -> None:
        if req.cfg.state != "hs" and not self.allow_jets:
            raise ValueError(f"request {req.rid}: jet-state requests need allow_jets")
        self.waiting.append(req)

    # -- admission -------------------------------------------------------------------------
    def admit(self) -> None:
        keep = []
        for req in self.waiting:
            if req.rid not in self.prepared:   # the host-side set-up is done once per request
                ga, f = self.backend.setup(req.cfg)
                ga.struct.hs_kf *= req.kf_scale
                need = self.backend.bytes(ga, self.precision)
                if need > self.hbm_budget:
                    raise ValueError(f"request {req.rid} needs {need} bytes, more than the whole budget")
                self.prepared[req.rid] = (ga, f, need)
            ga, f, need = self.prepared[req.rid]
            if self.used + need > self.hbm_budget:
                keep.append(req)
                continue
            m = self.backend.model(ga, f, self.precision)
            del self.prepared[req.rid]
            self.used += need
            self.peak_used = max(self.peak_used, self.used)
            cls = launch_class(req.cfg, getattr(ga.struct, "k_sigma", req.cfg.nk), self.precision, self.size_ratio)
            self.active.setdefault(cls, []).append(_Active(req, m, need, req.steps, self.now()))
        self.waiting = keep

    # -- one scheduling pass ----------------------------------------------------------------
    def round(self) -> bool:
        """Advance every launch class that is idle; a class whose batch is still running is left
        alone, so classes of different sizes never wait for one another.  Returns whether any
        class was handled."""
        progressed = False
        for cls in list(self.active):
            runs = self.active[cls]
            fl = self.inflight.get(cls)
            if fl is not None:
                b, n, members = fl
                if not b.done():
                    continue
                failed = {}
                try:
                    b.sync()
                except EpicError:
                    failed = self.backend.failures([r.model for r in members])
                del self.inflight[cls]
                progressed = True
                for q, r in enumerate(members):   # runs admitted meanwhile were not in this batch
                    if q in failed:
                        self._retire(cls, r, error=failed[q])
                        continue
                    r.remaining -= n
                    if r.remaining <= 0:
                        self._retire(cls, r)
            if not runs:
                continue
            ids = tuple(r.req.rid for r in runs)
            b = self.batches.get(cls)
            if b is None or b[1] != ids:          # a run joined or left: re-form the batch
                if b is not None:
                    b[0].close()
                b = (self.backend.batch([r.model for r in runs]), ids)
                self.batches[cls] = b
            n = min(self.round_steps, min(r.remaining for r in runs))
            b[0].run(n)
            self.inflight[cls] = (b[0], n, list(runs))
            progressed = True
        return progressed

    def _retire(self, cls, r: _Active, error: str | None = None) -> None:
        if error is None:
            f = r.model.download()
            res = RunResult(r.req.rid, (r.req.cfg.ni, r.req.cfg.nj, r.req.cfg.nk), r.req.steps, r.req.arrival, r.admitted,
                            self.now(), f if self.keep_fields else None, state_checksum(f))
        else:
            res = RunResult(r.req.rid, (r.req.cfg.ni, r.req.cfg.nj, r.req.cfg.nk), r.req.steps, r.req.arrival, r.admitted,
                            self.now(), None, float("nan"), error)
        self.results.append(res)
        self.active[cls].remove(r)
        b = self.batches.pop(cls, None)
        if b is not None:
            b[0].close()
        r.model.close()
        self.used -= r.bytes

    # -- the loop ---------------------------------------------------------------------------
    def serve(self, requests: list[RunRequest]) -> list[RunResult]:
        """Serve requests that arrive at their `arrival` times (seconds from now)."""
        pending = sorted(requests, key=lambda q: q.arrival)
        self.t0 = time.perf_counter()
        while pending or self.waiting or any(self.active.values()):
            t = self.now()
            while pending and pending[0].arrival <= t:
                self.submit(pending.pop(0))
            if self.waiting:
                self.admit()
            if any(self.active.values()):
                if not self.round():
                    time.sleep(0.0002)
            elif pending:
                time.sleep(max(0.0, min(0.01, pending[0].arrival - self.now())))
        for b, _ in self.batches.values():
            b.close()
        self.batches.clear()
        return sorted(self.results, key=lambda r: r.rid)


def poisson_requests(n: int, rate: float, seed: int, shapes: list[tuple], steps_range: tuple[int, int] | None = None,
                     dt_of=lambda shape: 300, jet_frac: float = 0.0, jet_dt_of=lambda shape: 60,
                     days_range: tuple[float, float] | None = None) -> list[RunRequest]:
    """n requests with seeded Poisson arrivals (mean `rate` per second), shapes drawn from
    `shapes` (ni, nj, nk), k_f scaled by 1 +/- 10%, and a duration either in steps (uniform in
    steps_range) or in simulated days (uniform in days_range, converted to steps of the request's
    time step); a fraction jet_frac of them (seeded) start from the balanced zonal jets on the
    constant-N^2 sounding with time step jet_dt_of(shape), the others from the Held-Suarez column
    with dt_of(shape)."""
    if (steps_range is None) == (days_range is None):
        raise ValueError("give one of steps_range and days_range")
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for q in range(n):
        t += float(rng.exponential(1.0 / rate))
        ni, nj, nk = shapes[int(rng.integers(len(shapes)))]
        dur = int(rng.integers(steps_range[0], steps_range[1] + 1)) if steps_range else float(rng.uniform(*days_range))
        kf = 1.0 + float(rng.uniform(-0.1, 0.1))
        if jet_frac > 0.0 and float(rng.uniform()) < jet_frac:
            cfg = HSConfig(ni=ni, nj=nj, nk=nk, dt=jet_dt_of((ni, nj, nk)), seed=1000 + q, profile=EPIC_PROFILE_N2, state="jet")
        else:
            cfg = HSConfig(ni=ni, nj=nj, nk=nk, dt=dt_of((ni, nj, nk)), seed=1000 + q)
        steps = dur if steps_range else max(1, int(round(dur * 86400.0 / cfg.dt)))
        out.append(RunRequest(q, cfg, steps, t, kf))
    return out


def latency_summary(results: list[RunResult]) -> dict:
    """p50/p99 time from arrival to completion over the runs that completed, and aggregate
    cell-steps/s over the makespan (runs ended by a model error count only up to their error)."""
    done = [r for r in results if r.error is None]
    lat = np.array([r.latency for r in done]) if done else np.array([np.nan])
    makespan = max(r.finished for r in results) - min(r.arrival for r in results)
    cells = sum(r.shape[0] * r.shape[1] * r.shape[2] * r.steps for r in done)
    return {"requests": len(results), "completed": len(done), "ended_by_model_error": len(results) - len(done),
            "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "makespan_s": makespan, "aggregate_cell_steps_per_s": cells / makespan,
            "errors": [{"rid": r.rid, "shape": list(r.shape), "steps": r.steps, "error": (r.error or "")[-160:]}
                       for r in results if r.error is not None]}
