"""Throughput of the GB300 EPIC timestep() on synthetic Held-Suarez states.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload ens64|hs64|hs128|hs256|hs512|jet256|jet256gg|jet256ggh2|hs128sa|jet128sa]
                    [--precision mixed|fast|fp64]
                    [--no-cpu-baseline] [--no-extras]

A step is one timestep(STEP_PROGS_AND_SYNC_DIAGS) of every grid in the workload.  metric =
cell-steps/s (cells = ni*nj*nk per grid).

Default workload ens64: an ensemble of 64 Held-Suarez members at 128 x 64 x 20, dt = 300 s,
each with its own noise seed and a +/-10% seeded drag rate k_f, advanced as one batch (every
kernel launched once for all members, one captured graph per step) in the mixed-precision
form.  The ensemble's state (64 x 54 MB) is far larger than the 129 MB L2, so no flush is
needed between steps.  Beside `value` the line reports the plain FP64 step of one member
shape and the mixed/FP64 ratio, the mixed form's error against FP64 after one simulated day,
and the serving loop's p50/p99 run latency on a seeded Poisson request stream.

value = cell-steps/s with the state resident in HBM, timed with CUDA events on the stream the
work runs on; e2e = the same metric through the C ABI with every member's state in pinned
host memory, uploaded and downloaded every step.

--impl reference times the reference's CPU implementation of the step (the oracle's
restatement, bit-identical to the reference build) on every host core as independent
replicas.  For N > 1 each GPU runs its own replica (the step does not shard).
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # name: (ni, nj, nk, dt)
    "hs64": (64, 32, 10, 300),
    "hs128": (128, 64, 20, 300),
    "hs256": (256, 128, 32, 60),
    "hs512": (512, 256, 40, 60),
    "jet256": (256, 128, 32, 60),  # balanced zonal jets on the constant-N^2 sounding
    "jet256gg": (256, 128, 32, 60),  # the same over the gas-giant lower boundary (gz_from_u)
    "jet256ggh2": (256, 128, 32, 60),  # and with the hydrogen-helium thermodynamics (thermo_setup's tables)
    "hs128sa": (128, 64, 20, 300),   # the Held-Suarez column with the Spalart-Allmaras DES closure (FP64)
    "jet128sa": (128, 64, 20, 300),  # the balanced jets with the Spalart-Allmaras DES closure (FP64)
    "ens64": (128, 64, 20, 300),   # per member; 64 members
}
ENSEMBLE = {"ens64": 64}
E2E_GROUPS = 8   # sub-batches of the end-to-end pipeline (copies of one overlap kernels of others)
# Serving stream: shapes and the time step each runs with for two simulated days (the mixed form
# from the Held-Suarez column at rest; a sweep of time steps per shape kept the largest that did
# not stop with non-monotonic GZ3 within two days for three seeds and k_f scaled by 0.9 and 1.1 --
# 128x64x32 stops at 120 s with the weaker drag, and at 100 s for some seeds).  256x128 and
# 512x256 with 20 or 32 layers stop within two days at every time step tried (down to 60 s and
# 30 s): left out.
SERVE_SHAPES = {(64, 32, 10): 300, (64, 32, 20): 240, (64, 32, 32): 300, (128, 64, 10): 240, (128, 64, 20): 120,
                (128, 64, 32): 90, (256, 128, 10): 120, (512, 256, 10): 60}
METRIC = "cell-steps/s"


ADVECTION = {"hsu": 0, "akima": 1}   # EPIC_ADV_HSU, EPIC_ADV_AKIMA
ADVECTION_NAME = {"hsu": "Hsu-Konor-Arakawa advection", "akima": "Akima advection"}


def _workload_cfg(name, seed=0, advection="hsu"):
    from epic_gb300 import EPIC_PROFILE_N2, HSConfig
    ni, nj, nk, dt = WORKLOADS[name]
    turb = name.endswith("sa")
    h2 = {"x_h2": 0.864, "x_he": 0.136} if name.endswith("h2") else {}
    if name.startswith("jet"):
        return HSConfig(ni=ni, nj=nj, nk=nk, dt=dt, seed=seed, advection_scheme=ADVECTION[advection], profile=EPIC_PROFILE_N2,
                        state="jet", gas_giant="gg" in name, turbulence=turb, **h2)
    return HSConfig(ni=ni, nj=nj, nk=nk, dt=dt, seed=seed, advection_scheme=ADVECTION[advection], turbulence=turb)


def algorithmic_bytes_per_step(cfg, word=8):
    """Compulsory HBM traffic of one AB3 step: U, V, HDRY, THETA and the two older tendency
    planes of U and V read once; U, V, HDRY, THETA and the new tendencies written once."""
    return 14 * word * cfg.ni * (cfg.nj + 1) * cfg.nk


# ---------------------------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------------------------

class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                                          "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.25)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        if not self.path or not os.path.exists(self.path):
            return out
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        if sm:
            out.update(sm_mhz=statistics.median(sm), sm_max_mhz=max(mx), reasons=sorted(reasons), samples=len(sm))
        return out


# ---------------------------------------------------------------------------------------------
# CPU side: the oracle's restatement of the reference step
# ---------------------------------------------------------------------------------------------

def kf_scales(n, seed=7):
    """The ensemble's drag-rate factors: member q runs with k_f * (1 + U[-0.1, 0.1]), drawn in order."""
    import numpy as np
    rng = np.random.default_rng(seed)
    return [1.0 + float(rng.uniform(-0.1, 0.1)) for _ in range(n)]


def _cpu_worker(name, jobs, nsteps, warm, advection, q):
    """Step each (seed, k_f factor) grid of `jobs` in turn on this core: set-up, priming and
    `warm` steps untimed, then `nsteps` timed steps; reports the summed timed seconds."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from oracle_lib import Port
    from epic_gb300 import EPIC_SYNC_DIAGS_ONLY, hs_setup
    total = 0.
    for seed, scale in jobs:
        cfg = _workload_cfg(name, seed, advection)
        ga, f = hs_setup(cfg)
        ga.struct.hs_kf *= scale
        p = Port(ga)
        p.upload(f)
        p.timestep(EPIC_SYNC_DIAGS_ONLY)
        p.run(warm)
        t0 = time.perf_counter()
        p.run(nsteps)
        total += time.perf_counter() - t0
    q.put(total)


def cpu_reference(name, nsteps, warm, procs, advection="hsu", grids=1, scales=None):
    """Aggregate cell-steps/s of the reference step (the oracle's restatement, single-threaded
    like the reference) over `grids` grids spread round-robin over `procs` worker processes, one
    per host core: grid g has noise seed g and k_f factor scales[g].  The rate is the cells of
    every grid times nsteps over the slowest worker's timed seconds."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from oracle_lib import build_port
    build_port()
    scales = scales or [1.0] * grids
    nw = max(1, min(procs, grids))
    jobs = [[] for _ in range(nw)]
    for g in range(grids):
        jobs[g % nw].append((g, scales[g]))
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_cpu_worker, args=(name, j, nsteps, warm, advection, q)) for j in jobs]
    for p in ps:
        p.start()
    times = [q.get(timeout=3600) for _ in ps]
    for p in ps:
        p.join()
    cfg = _workload_cfg(name)
    wall = max(times)
    return grids * cfg.cells * nsteps / wall, wall


def host_link_gbs(torch, nbytes: int = 1 << 30, reps: int = 3) -> dict:
    """Pinned host <-> device copy bandwidth of this machine (GB/s): one direction at a time, then both
    at once on two streams -- what bounds the end-to-end number, whose state crosses twice a step."""
    h_up = torch.empty(nbytes // 8, dtype=torch.float64, pin_memory=True)
    h_dn = torch.empty_like(h_up, pin_memory=True)
    d_up = torch.empty(nbytes // 8, dtype=torch.float64, device="cuda")
    d_dn = torch.empty_like(d_up)
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) / reps

    def both():
        with torch.cuda.stream(s1):
            d_up.copy_(h_up, non_blocking=True)
        with torch.cuda.stream(s2):
            h_dn.copy_(d_dn, non_blocking=True)

    t_up = timed(lambda: d_up.copy_(h_up, non_blocking=True))
    t_dn = timed(lambda: h_dn.copy_(d_dn, non_blocking=True))
    t_both = timed(both)
    del h_up, h_dn, d_up, d_dn
    return {"h2d": nbytes / t_up / 1e9, "d2h": nbytes / t_dn / 1e9, "both_directions": 2 * nbytes / t_both / 1e9}


def workload_config(args, cfg, nmem, ws):
    """The `config` object of both arms' lines: the workload only (shape, members, time step,
    schemes, state), so that the GPU arm and the reference arm name the same one."""
    state = ("6 seeded Gaussian zonal jets (50-150 m/s, centres -70..70 deg, widths 3-8 deg) in gradient-wind balance "
             "on a constant N^2 = 1e-4 s^-2 sounding (isothermal at 200 K above), 1% seeded vorticity perturbation"
             if cfg.state == "jet" else "horizontally uniform HS equilibrium column at rest + seeded 0.1 K theta noise")
    # u, v (AB3: one plane each), three tendency planes each, 20 single fields
    state_gb = nmem * 28 * 8 * (cfg.ni + 2) * (cfg.nj + 3) * (cfg.nk + 2) / 1e9
    if nmem > 1:
        what = (f"ensemble of {nmem} Held-Suarez members {cfg.ni}x{cfg.nj}x{cfg.nk}, dt={cfg.dt}s, AB3, "
                f"{ADVECTION_NAME[args.advection]}, nu4=0.5 max, seeded 0.1 K noise and +/-10% k_f per member")
    else:
        what = (("Zonal jets on the Held-Suarez planet " if cfg.state == "jet" else "Held-Suarez ") +
                ("over the gas-giant lower boundary (GZ_SURFACE from gz_from_u) " if cfg.gas_giant else "") +
                ("with the hydrogen-helium thermodynamics (x_h2 0.864, x_he 0.136, normal hydrogen) " if cfg.x_h2 > 0 else "") +
                ("with the Spalart-Allmaras DES turbulence closure " if cfg.turbulence else "") +
                f"{cfg.ni}x{cfg.nj}x{cfg.nk}, dt={cfg.dt}s, AB3, {ADVECTION_NAME[args.advection]}, nu4=0.5 max")
    return {"workload": what, "ni": cfg.ni, "nj": cfg.nj, "nk": cfg.nk, "dt": cfg.dt, "members": nmem,
            "advection": args.advection, "parallelism": f"replicas{ws}", "state": state,
            "l2": f"every step reads and writes the whole state, {state_gb:.2f} GB of binary64 arrays "
                  + ("> 129 MB L2; no flush needed" if state_gb > 0.129 else "(fits in the 129 MB L2; no flush)")}


# ---------------------------------------------------------------------------------------------
# GPU side
# ---------------------------------------------------------------------------------------------

def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def run_gpu(args):
    import torch
    from epic_gb300 import EPIC_PREC_FP64, EPIC_PREC_MIXED, EPIC_SYNC_DIAGS_ONLY, Model, hs_setup
    ws, rank, local = _dist()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    cfg = _workload_cfg(args.workload, seed=rank, advection=args.advection)
    ga, f = hs_setup(cfg)
    model = Model(ga, _prec(args.precision))
    model.upload(f)
    model.timestep(EPIC_SYNC_DIAGS_ONLY)
    stream = torch.cuda.ExternalStream(model.stream)
    for _ in range(args.warmup):
        model.run(1)
    model.sync()

    def barrier():
        torch.cuda.synchronize()
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()

    # device-resident throughput
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    with ClockSampler(local) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            model.run(1)
        ev1.record(stream)
        ev1.synchronize()
    model.sync()
    barrier()
    ms = ev0.elapsed_time(ev1)
    if ws > 1:
        import torch.distributed as dist
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    ms_step = ms / args.steps
    value = ws * cfg.cells * args.steps / (ms / 1e3)
    clocks = clk.summary()

    # dominant kernel, timed alone with events: the vertical Hsu advection stage
    roof = kernel_roofline(model, cfg, stream, torch)

    # end to end through the C ABI with pinned host state
    host = model.download().copy(pinned=True)
    e2e_steps = max(1, min(args.steps, 5))
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        model.step_host(host, 1, prime=False)
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    e2e_val = ws * cfg.cells / e2e_s
    launches = model.kernels_per_step * args.steps

    out = None
    if rank == 0:
        peaks = _peaks()
        out = {
            "metric": METRIC, "value": value, "unit": "cell-steps/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f32+f64", "data": "synthetic",
            "config": workload_config(args, cfg, 1, ws),
            "form": args.precision,
            "clocks": clocks,
            "e2e": {"value": e2e_val, "unit": "cell-steps/s", "h2d_bytes_per_step": host.nbytes,
                    "d2h_bytes_per_step": host.nbytes},
            "gpu_launches": launches,
            "roofline": roof,
            "step_roofline": {"bound": "hbm", "algorithmic_bytes_per_step": algorithmic_bytes_per_step(cfg),
                              "achieved_gbs": algorithmic_bytes_per_step(cfg) / (ms_step / 1e3) / 1e9,
                              "peak_gbs": peaks.get("hbm_gbs")},
        }
        if peaks.get("hbm_gbs"):
            out["step_roofline"]["frac"] = out["step_roofline"]["achieved_gbs"] / peaks["hbm_gbs"]
    model.close()
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return out


def _members(cfg, n, precision, torch_seed=7):
    """n ensemble members of one shape: member q has noise seed q and k_f scaled by 1 +/- 10%."""
    from epic_gb300 import HSConfig, Model, hs_setup
    out = []
    for q, scale in enumerate(kf_scales(n, torch_seed)):
        ga, f = hs_setup(HSConfig(ni=cfg.ni, nj=cfg.nj, nk=cfg.nk, dt=cfg.dt, seed=q, advection_scheme=cfg.advection_scheme))
        ga.struct.hs_kf *= scale
        m = Model(ga, precision)
        m.upload(f)
        out.append(m)
    return out


def single_rate(cfg, precision, steps, torch):
    """cell-steps/s of one model stepped alone (graph replay), timed with events on its stream."""
    from epic_gb300 import EPIC_SYNC_DIAGS_ONLY, Model, hs_setup
    ga, f = hs_setup(cfg)
    m = Model(ga, precision)
    m.upload(f)
    m.timestep(EPIC_SYNC_DIAGS_ONLY)
    m.run(3)
    m.sync()
    st = torch.cuda.ExternalStream(m.stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    m.run(steps)
    e1.record(st)
    e1.synchronize()
    m.sync()
    ms = e0.elapsed_time(e1) / steps
    m.close()
    return {"value": cfg.cells / (ms / 1e3), "ms_per_step": ms}


def _prec(name):
    from epic_gb300 import EPIC_PREC_FP64, EPIC_PREC_MIXED, EPIC_PREC_MIXED_FAST
    return {"fp64": EPIC_PREC_FP64, "mixed": EPIC_PREC_MIXED, "fast": EPIC_PREC_MIXED_FAST}[name]


def mixed_error(torch, precision, advection="hsu"):
    """Per-prognostic relative L2 of a mixed form against FP64 after one simulated day
    (288 steps of 300 s) at 64x32x10, from a state spun up for 10 days in FP64, and from rest
    (both the spin-up and the day use the given advection scheme)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from compare import PROGNOSTIC, field_errors
    from epic_gb300 import EPIC_PREC_FP64, EPIC_SYNC_DIAGS_ONLY, HSConfig, Model, hs_setup
    ga, f = hs_setup(HSConfig(ni=64, nj=32, nk=10, dt=300, seed=0, advection_scheme=ADVECTION[advection]))
    out = {}
    for label, spin in (("after_10_day_spin_up", 2880), ("from_rest", 0)):
        start = f
        if spin:
            m = Model(ga, EPIC_PREC_FP64)
            m.upload(f)
            m.timestep(EPIC_SYNC_DIAGS_ONLY)
            m.run(spin)
            m.sync()
            start = m.download()
            m.close()
        res = []
        for prec in (EPIC_PREC_FP64, precision):
            m = Model(ga, prec)
            m.upload(start)
            if not spin:
                m.timestep(EPIC_SYNC_DIAGS_ONLY)
            m.run(288)
            m.sync()
            res.append(m.download())
            m.close()
        e = field_errors(res[1], res[0], PROGNOSTIC)
        out[label] = {k: v[0] for k, v in e.items()}
    out["case"] = (f"64x32x10, dt=300 s, {ADVECTION_NAME[advection]}, 1 simulated day (288 steps), relative L2 per "
                   f"prognostic vs the FP64 form")
    return out


_ENSEMBLE_RUNS = {}


def _ensemble_day(cfg, nmem, precision, steps):
    """Prognostic fields of every member after `steps` steps from rest, stepped as one batch
    (the launch shapes of the timed ensemble: with 64 members of 128x64x20 the meridional Hsu
    passes of UNITY and HDRY take the fused march).  Cached per form: the FP64 run serves every
    form's comparison."""
    import numpy as np
    from epic_gb300 import EPIC_SYNC_DIAGS_ONLY, Batch
    key = (cfg.ni, cfg.nj, cfg.nk, cfg.dt, cfg.advection_scheme, nmem, precision, steps)
    if key not in _ENSEMBLE_RUNS:
        members = _members(cfg, nmem, precision, torch_seed=7)
        b = Batch(members)
        b.timestep(EPIC_SYNC_DIAGS_ONLY)
        b.run(steps)
        b.sync()
        out = []
        for m in members:
            f = m.download()
            out.append({k: np.array(f.arrays[k], copy=True) for k in ("u", "v", "hdry", "theta")})
        b.close()
        for m in members:
            m.close()
        _ENSEMBLE_RUNS[key] = out
    return _ENSEMBLE_RUNS[key]


def ensemble_error(torch, precision, cfg, nmem=64, steps=288):
    """The ensemble error at the member shape, on the timed ensemble itself: nmem members
    (ensemble_rate's seeds and k_f perturbations) stepped one simulated day from rest as a batch
    in the given form and in FP64.  Reported per prognostic: relative L2 of the ensemble mean and
    of the ensemble spread (standard deviation over members) against FP64's, and the largest and
    the median per-member relative L2 (relative L2 over each member's interior cells)."""
    import numpy as np
    from epic_gb300 import EPIC_PREC_FP64
    from epic_gb300.abi import Layout
    ref = _ensemble_day(cfg, nmem, EPIC_PREC_FP64, steps)
    got = _ensemble_day(cfg, nmem, precision, steps)
    L = Layout(cfg.ni, cfg.nj, cfg.nk)
    kinds = {"u": "uv", "v": "vv", "hdry": "h", "theta": "h"}
    out = {"mean": {}, "spread": {}, "member_max": {}, "member_median": {}, "max_abs_over_max": {}}
    for k in ("u", "v", "hdry", "theta"):
        plane = (lambda a: a[0]) if k in ("u", "v") else (lambda a: a)
        a = np.stack([L.interior(plane(g[k]), kinds[k]) for g in got])
        r = np.stack([L.interior(plane(f[k]), kinds[k]) for f in ref])
        out["mean"][k] = float(np.linalg.norm(a.mean(0) - r.mean(0)) / np.linalg.norm(r.mean(0)))
        out["spread"][k] = float(np.linalg.norm(a.std(0) - r.std(0)) / np.linalg.norm(r.std(0)))
        per = [float(np.linalg.norm(x - y) / np.linalg.norm(y)) for x, y in zip(a, r)]
        out["member_max"][k] = max(per)
        out["member_median"][k] = float(np.median(per))
        out["max_abs_over_max"][k] = float(np.abs(a - r).max() / np.abs(r).max())
    out["case"] = (f"{nmem} members {cfg.ni}x{cfg.nj}x{cfg.nk}, dt={cfg.dt} s, {steps} steps (1 simulated day) from rest, "
                   f"batched as in the timed run, relative L2 over interior cells vs the FP64 members")
    return out


def cfg2_error(precision, steps=240):
    """The mixed-precision configuration's own shape, 512x256x40 (the 512x512 tensor-core filter
    operator), from rest at dt = 60 s for `steps` steps -- the FP64 run of this state stops with
    non-monotonic GZ3 after ~288 steps at dt 60 and within the first steps at dt 150 -- against the
    FP64 form: relative L2 over interior cells and max |error| / max |FP64| per prognostic."""
    import numpy as np
    from epic_gb300 import EPIC_PREC_FP64, EPIC_SYNC_DIAGS_ONLY, HSConfig, Model, hs_setup
    from epic_gb300.abi import Layout
    ga, f = hs_setup(HSConfig(ni=512, nj=256, nk=40, dt=60, seed=0))
    res = []
    for prec in (EPIC_PREC_FP64, precision):
        m = Model(ga, prec)
        m.upload(f)
        m.timestep(EPIC_SYNC_DIAGS_ONLY)
        m.run(steps)
        m.sync()
        res.append(m.download())
        m.close()
    L = Layout(512, 256, 40)
    out = {"rel_l2": {}, "max_abs_over_max": {}}
    for k, kind in (("u", "uv"), ("v", "vv"), ("hdry", "h"), ("theta", "h")):
        pick = (lambda x: x.wind(k)) if k in ("u", "v") else (lambda x: x.arrays[k])
        a, r = L.interior(pick(res[1]), kind), L.interior(pick(res[0]), kind)
        out["rel_l2"][k] = float(np.linalg.norm(a - r) / np.linalg.norm(r))
        out["max_abs_over_max"][k] = float(np.abs(a - r).max() / np.abs(r).max())
    out["case"] = f"512x256x40, dt=60 s, {steps} steps ({steps * 60 / 3600:.0f} h) from rest, vs the FP64 form"
    return out


def serving_accuracy(reqs, res, precision, max_runs=6, max_ni=128):
    """The mixed form's error against FP64 on the stream's own requests: the first `max_runs`
    completed requests with ni <= max_ni, each run alone in both forms for its steps (a served run
    equals itself run alone bit for bit, tests/test_gpu_serving.py); relative L2 over interior
    cells per prognostic, the largest over those runs."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from compare import PROGNOSTIC, field_errors
    from epic_gb300 import EPIC_PREC_FP64, EPIC_SYNC_DIAGS_ONLY, Model, hs_setup
    done = {r.rid for r in res if r.error is None}
    picked = [q for q in reqs if q.rid in done and q.cfg.ni <= max_ni][:max_runs]
    worst = {k: 0.0 for k in PROGNOSTIC}
    runs = []
    for q in picked:
        ga, f = hs_setup(q.cfg)
        ga.struct.hs_kf *= q.kf_scale
        out = []
        for prec in (EPIC_PREC_FP64, precision):
            m = Model(ga, prec)
            m.upload(f)
            m.timestep(EPIC_SYNC_DIAGS_ONLY)
            m.run(q.steps)
            m.sync()
            out.append(m.download())
            m.close()
        e = {k: v[0] for k, v in field_errors(out[1], out[0], PROGNOSTIC).items()}
        runs.append({"rid": q.rid, "shape": [q.cfg.ni, q.cfg.nj, q.cfg.nk], "state": q.cfg.state, "steps": q.steps,
                     "days": q.steps * q.cfg.dt / 86400.0, "rel_l2": e})
        for k in worst:
            worst[k] = max(worst[k], e[k])
    return {"max_rel_l2": worst, "runs": runs,
            "case": f"the first {len(picked)} completed requests with ni <= {max_ni}, each run alone in FP64 and the "
                    "mixed form for its whole duration; relative L2 over interior cells vs FP64"}


def serving_summary(precision, seed=3, nreq=24, jet_frac=0.0):
    """The serving loop on a seeded Poisson stream (20 requests/s) of runs of the shapes of
    SERVE_SHAPES, each lasting U[0.25, 2] simulated days: Held-Suarez runs, and a fraction
    jet_frac of zonal-jet runs (dt 60 s)."""
    from epic_gb300.serving import RunServer, latency_summary, poisson_requests
    reqs = poisson_requests(nreq, 20.0, seed, sorted(SERVE_SHAPES), dt_of=lambda s: SERVE_SHAPES[s], days_range=(0.25, 2.0),
                            jet_frac=jet_frac, jet_dt_of=lambda s: 60)
    res = RunServer(hbm_budget=40 << 30, precision=precision, round_steps=16).serve(reqs)
    out = latency_summary(res)
    out["accuracy"] = serving_accuracy(reqs, res, precision)
    states = "Held-Suarez column at rest with seeded theta noise"
    if jet_frac > 0.0:
        states += (f"; {sum(r.cfg.state == 'jet' for r in reqs)} of the {nreq} requests in the balanced zonal-jet state on "
                   "the constant-N^2 sounding at dt 60 s")
    out.update({"arrivals": f"Poisson, 20 requests/s, seed {seed}", "states": states,
                "shapes": [list(k) + [v] for k, v in sorted(SERVE_SHAPES.items())],
                "durations": "uniform 0.25-2 simulated days (steps = days * 86400 / dt)", "hbm_budget_gb": 40,
                "batching": "runs of one launch class (layers, schemes, form, filter path) share a batch, sizes and dt may differ",
                "note": "256x128 and 512x256 with 20 or 32 layers are left out: from this state they stop with "
                        "non-monotonic GZ3 within two days at every time step tried"})
    return out


def ensemble_rate(cfg, nmem, precision, args, torch, rank):
    """Cell-steps/s of one ensemble in a given form (tuned, primed, timed like the headline)."""
    from epic_gb300 import EPIC_SYNC_DIAGS_ONLY, Batch
    members = _members(cfg, nmem, precision, torch_seed=7 + rank)
    starts = [m.download() for m in members]
    batch = Batch(members)
    if not args.no_tune:
        batch.timestep(EPIC_SYNC_DIAGS_ONLY)
        batch.autotune(trial_steps=2)
        batch.sync()
        for m, f in zip(members, starts):
            m.upload(f)
    batch.timestep(EPIC_SYNC_DIAGS_ONLY)
    for _ in range(args.warmup):
        batch.run(1)
    batch.sync()
    stream = torch.cuda.ExternalStream(batch.stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        batch.run(1)
    e1.record(stream)
    e1.synchronize()
    batch.sync()
    ms = e0.elapsed_time(e1)
    batch.close()
    for m in members:
        m.close()
    return {"value": nmem * cfg.cells * args.steps / (ms / 1e3), "ms_per_step": ms / args.steps}


def run_gpu_ensemble(args):
    import torch
    from epic_gb300 import EPIC_IO_ALL, EPIC_IO_STATE, EPIC_PREC_FP64, EPIC_PREC_MIXED, EPIC_SYNC_DIAGS_ONLY, Batch
    ws, rank, local = _dist()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    precision = _prec(args.precision)
    cfg = _workload_cfg(args.workload, advection=args.advection)
    nmem = args.members or ENSEMBLE[args.workload]
    members = _members(cfg, nmem, precision, torch_seed=7)
    starts = [m.download() for m in members]
    batch = Batch(members)
    tuning = None
    if not args.no_tune:
        # launch shapes: autotuned on this batch (primed), then every member goes back to its
        # initial state
        batch.timestep(EPIC_SYNC_DIAGS_ONLY)
        tuning = batch.autotune(trial_steps=2)
        batch.sync()
        for m, f in zip(members, starts):
            m.upload(f)
    batch.timestep(EPIC_SYNC_DIAGS_ONLY)
    for _ in range(args.warmup):
        batch.run(1)
    batch.sync()
    stream = torch.cuda.ExternalStream(batch.stream)

    def barrier():
        torch.cuda.synchronize()
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()

    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    with ClockSampler(local) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            batch.run(1)
        ev1.record(stream)
        ev1.synchronize()
    batch.sync()
    barrier()
    ms = ev0.elapsed_time(ev1)
    if ws > 1:
        import torch.distributed as dist
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    ms_step = ms / args.steps
    cells = nmem * cfg.cells
    value = ws * cells * args.steps / (ms / 1e3)
    clocks = clk.summary()
    launches = batch.kernels_per_step * args.steps

    # the largest stage of the step (the pressure gradient, 13-15% of it; k_pgrad_lat and
    # k_pgrad_lon are among the top kernels of the launch list) and the vertical integration
    # feeding it
    roof = batch_roofline(batch, cfg, nmem, stream, torch, stage=12)
    roof_column = batch_roofline(batch, cfg, nmem, stream, torch, stage=19)

    # end to end: every member's prognostic state (u, v, the tendency planes, hdry, theta) uploaded
    # from pinned host memory and downloaded, each step; and, beside it, every array of the state
    hosts = [m.download().copy(pinned=True) for m in members]
    e2e_steps = max(1, min(args.steps, 6))

    def e2e_run(io):
        batch.step_host(hosts, 1, groups=E2E_GROUPS, io=io)   # the first call builds the sub-batch graphs
        barrier()
        t0 = time.perf_counter()
        batch.step_host(hosts, e2e_steps, groups=E2E_GROUPS, io=io)
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) / e2e_steps

    e2e_s = e2e_run(EPIC_IO_STATE)
    e2e_val = ws * cells / e2e_s
    e2e_all_s = e2e_run(EPIC_IO_ALL)
    host_bytes = sum(h.nbytes for h in hosts)
    state_bytes = sum(h.state_nbytes for h in hosts)
    link = host_link_gbs(torch)
    state_gb = sum(m.device_bytes for m in members) / 1e9
    batch.close()
    for m in members:
        m.close()

    out = None
    if rank == 0:
        peaks = _peaks()
        out = {
            "metric": METRIC, "value": value, "unit": "cell-steps/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if precision == EPIC_PREC_FP64 else "f32+f64", "data": "synthetic",
            "config": workload_config(args, cfg, nmem, ws),
            "form": f"{args.precision} precision form, one launch per kernel for all members under a captured CUDA graph",
            "launch_shapes": {"autotuned": tuning,
                              "groups": ["uv_core", "pgrad", "hsu_meridional", "hyperviscosity", "diagnostics",
                                         "update", "column", "pointwise", "row_filter",
                                         "hsu_meridional_form (1 fused march, 2 four passes)"]},
            "clocks": clocks,
            "e2e": {"value": e2e_val, "unit": "cell-steps/s", "h2d_bytes_per_step": state_bytes, "d2h_bytes_per_step": state_bytes,
                    "ms_per_step": e2e_s * 1e3, "host_link_gbs": link,
                    "link_bound_ms_per_step": 2e3 * state_bytes / (link["both_directions"] * 1e9) if link.get("both_directions") else None,
                    "all_arrays": {"value": ws * cells / e2e_all_s, "ms_per_step": e2e_all_s * 1e3, "h2d_bytes_per_step": host_bytes,
                                   "d2h_bytes_per_step": host_bytes,
                                   "link_bound_ms_per_step": 2e3 * host_bytes / (link["both_directions"] * 1e9) if link.get("both_directions") else None},
                    "note": "Batch.step_host with EPIC_IO_STATE: every step uploads each member's prognostic arrays (u, v, the three "
                            "AB3 tendency planes of each, hdry, theta) from pinned host memory, steps, and downloads them, in 8 "
                            "sub-batches on their own streams (copies of one overlap the kernels of the others); the diagnostics "
                            "stay on the device, which recomputes them. all_arrays moves every array of the state each way "
                            "(EPIC_IO_ALL). host_link_gbs: one pinned copy alone in each direction and both at once on this box"},
            "gpu_launches": launches,
            "roofline": roof,
            "roofline_store_pgrad_vars": roof_column,
            "step_roofline": {"bound": "hbm", "algorithmic_bytes_per_step": nmem * algorithmic_bytes_per_step(cfg),
                              "achieved_gbs": nmem * algorithmic_bytes_per_step(cfg) / (ms_step / 1e3) / 1e9,
                              "peak_gbs": peaks.get("hbm_gbs")},
        }
        if peaks.get("hbm_gbs"):
            out["step_roofline"]["frac"] = out["step_roofline"]["achieved_gbs"] / peaks["hbm_gbs"]
        if not args.no_extras:
            fp64 = single_rate(cfg, EPIC_PREC_FP64, args.steps, torch)
            mixed = single_rate(cfg, precision, args.steps, torch)
            out["fp64_single"] = dict(fp64, note=f"plain FP64 timestep of one {cfg.ni}x{cfg.nj}x{cfg.nk} grid")
            out["mixed_single"] = dict(mixed, note=f"{args.precision} form, one {cfg.ni}x{cfg.nj}x{cfg.nk} grid")
            out["batched_over_fp64_single"] = value / ws / fp64["value"]
            if precision != EPIC_PREC_FP64:
                out["mixed_error"] = mixed_error(torch, precision, args.advection)
                out["cfg2_error"] = cfg2_error(precision)
                out["ensemble_error"] = ensemble_error(torch, precision, cfg, nmem)
            if args.precision == "mixed":
                # the faster form that keeps the vertical integration and pressure gradient in FP32
                fast = ensemble_rate(cfg, nmem, _prec("fast"), args, torch, rank)
                out["mixed_fast"] = dict(fast, error=mixed_error(torch, _prec("fast"), args.advection),
                                         ensemble_error=ensemble_error(torch, _prec("fast"), cfg, nmem),
                                         note="EPIC_PREC_MIXED_FAST ensemble, same workload and timing")
            out["serving"] = serving_summary(precision)
            out["serving_with_jets"] = serving_summary(precision, seed=11, jet_frac=0.5)
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()
    return out


# Stages timed for the roofline: (stage, kernels, algorithmic 8-byte field passes per cell, note)
ROOF_STAGES = {
    19: ("store_pgrad_vars before the pressure gradient (the column tile of the form + k_pgrad_dzdt) over all members", 20,
        "THETA, P3, P2, THETA2, GZ3, W3, H3 read and T3, EXNER3, RHO3, T2, RHO2, GZ3, MONT3, DZDT3 written by the "
        "column tile; U, V, GZ3, DZDT3 read and DZDT3 written by the horizontal part; bound by load latency and "
        "the FP64 hydrostatic sum, not by HBM"),
    12: ("uv_pgrad_finite_volume (k_gz_pole_rows + k_pgrad_lon + k_pgrad_lat) over all members", 7,
         "GZ3, P2, RHO3 read and DUDT, DVDT read and written; stencils of 18-24 loads per cell from L1/L2 plus ~300 "
         "FP32/integer operations: issue- and latency-bound, not HBM-bound"),
}


# DRAM traffic per member of each roofline stage: dram__bytes_read.sum + dram__bytes_write.sum of
# the stage's kernels from one ncu capture of an 8-member launch at 128x64x20 (cold L2; writes
# still resident in L2 when a kernel ends are not counted), divided by 8
# (profiles/traffic_stages_mixed_ensemble8_128x64x20.md).  Scaled by the members of the launch.
ROOF_TRAFFIC_PER_MEMBER = {19: 184.7e6 / 8, 12: 86.4e6 / 8}
# Issue fraction of each roofline stage (smsp__issue_active, duration-weighted over the stage's
# kernels, one ncu capture of an 8-member step at 128x64x20,
# profiles/kernels_hbm_issue_mixed_ensemble8_128x64x20.md): the bound these kernels meet, beside
# the HBM fraction they do not
ROOF_ISSUE = {12: 0.826, 19: 0.609}
ROOF_TRAFFIC_SHAPE = (128, 64, 20)


def batch_roofline(batch, cfg, nmem, stream, torch, stage=19):
    """One stage of the step over all members, timed with CUDA events on the batch stream after
    a warm-up call.  Algorithmic bytes per launch: the stage's field passes (ROOF_STAGES) of
    8-byte values over ni*(nj+1)*nk cells per member.  Stage 19 (store_pgrad_vars feeding the
    pressure gradient) holds the largest kernel of the mixed step, k_pgrad_vars_column_acc."""
    peaks = _peaks()
    label, passes, note = ROOF_STAGES[stage]
    n = 5
    batch.run_stage(stage)
    batch.sync()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(n):
        batch.run_stage(stage)
    e1.record(stream)
    e1.synchronize()
    batch.sync()
    dur = e0.elapsed_time(e1) / n / 1e3
    alg = passes * 8 * cfg.ni * (cfg.nj + 1) * cfg.nk * nmem
    ach = alg / dur / 1e9
    traffic = None
    if (cfg.ni, cfg.nj, cfg.nk) == ROOF_TRAFFIC_SHAPE and stage in ROOF_TRAFFIC_PER_MEMBER:
        traffic = ROOF_TRAFFIC_PER_MEMBER[stage] * nmem
    return {"kernel": label, "bound": "hbm", "achieved": ach, "peak": peaks["hbm_gbs"], "unit": "GB/s",
            "frac": ach / peaks["hbm_gbs"], "peak_source": peaks["source"] + " (burst copy)", "algorithmic_bytes": alg,
            "launch_ms": dur * 1e3, "traffic": traffic,
            "issue_frac": ROOF_ISSUE.get(stage),
            "issue_source": "ncu smsp__issue_active of the stage's kernels, duration-weighted, one 8-member step at "
                            "128x64x20 (a constant of that capture)" if stage in ROOF_ISSUE else None,
            "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of the stage's kernels, one 8-member launch "
                              "at 128x64x20 scaled by members" if traffic else None, "note": note}


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        d["source"] = "measured"
        return d
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "source": "fallback"}


def kernel_roofline(model, cfg, stream, torch):
    """Stage 6 (advection: three passes of the grid's scheme, Hsu or Akima) timed alone.

    Algorithmic bytes per launch: each advected field (unity, THETA, HDRY) is read and written
    once, plus U, V, W3 read once: 6 reads + 3 writes of one FP64 3-D field
    (ni*(nj+1)*nk cells)."""
    peaks = _peaks()
    n = 5
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    state = model.download()
    model.run_stage(6)
    model.sync()
    model.upload(state)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(n):
        model.run_stage(6)
    e1.record(stream)
    e1.synchronize()
    model.upload(state)
    model.sync()
    dur = e0.elapsed_time(e1) / n / 1e3
    cells = cfg.ni * (cfg.nj + 1) * cfg.nk
    alg = 9 * 8 * cells
    ach = alg / dur / 1e9
    scheme = "akima_advection" if cfg.advection_scheme == ADVECTION["akima"] else "hsu_advection"
    return {"kernel": f"advection ({scheme} of unity, THETA, HDRY)", "bound": "hbm", "achieved": ach,
            "peak": peaks["hbm_gbs"], "unit": "GB/s", "frac": ach / peaks["hbm_gbs"],
            "peak_source": peaks["source"] + " (burst copy)", "algorithmic_bytes": alg, "launch_ms": dur * 1e3,
            "traffic": None}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="ens64", choices=sorted(WORKLOADS))
    ap.add_argument("--no-extras", action="store_true", help="skip the FP64/mixed single-grid, error and serving figures")
    ap.add_argument("--members", type=int, default=None, help="ensemble size (profiling runs use a smaller ensemble)")
    ap.add_argument("--no-tune", action="store_true", help="keep the built-in launch shapes (profiling runs)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-steps", type=int, default=100)
    ap.add_argument("--precision", default=None, choices=["fp64", "mixed", "fast"])
    ap.add_argument("--advection", default="hsu", choices=sorted(ADVECTION),
                    help="THETA/HDRY advection scheme (the Held-Suarez default is hsu)")
    args = ap.parse_args()
    if args.precision is None:
        args.precision = "mixed" if args.workload in ENSEMBLE else "fp64"
    ws, rank, _ = _dist()

    if args.impl == "reference":
        if rank != 0:
            return
        procs = os.cpu_count() or 1
        cfg = _workload_cfg(args.workload, advection=args.advection)
        nmem = (args.members or ENSEMBLE[args.workload]) if args.workload in ENSEMBLE else 1
        # the ensemble: the GPU arm's members (seeds, k_f factors) over every host core; a single
        # grid: one replica per host core (the reference is single-threaded)
        grids = nmem if nmem > 1 else procs
        val, wall = cpu_reference(args.workload, args.steps, args.warmup, procs, args.advection, grids=grids,
                                  scales=kf_scales(nmem) if nmem > 1 else None)
        line = {"impl": "reference", "metric": METRIC, "value": val, "unit": "cell-steps/s", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": wall / args.steps * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": workload_config(args, cfg, nmem, args.gpus),
                "form": "reference CPU step (FP64, single-threaded) on the host cores",
                "cpu_baseline": {"value": val, "unit": "cell-steps/s", "cores": min(procs, grids), "kind": "port",
                                 "sample": f"{grids} grids of the workload round-robin over {min(procs, grids)} worker "
                                           f"processes (one per host core), {args.warmup} untimed + {args.steps} timed steps "
                                           f"each, with the oracle's restatement of the step (bit-identical to the "
                                           f"reference build, which needs the reference tree to compile); rate = cells of "
                                           f"every grid x steps / slowest worker's timed seconds"},
                "e2e": {"value": val, "unit": "cell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    out = run_gpu_ensemble(args) if args.workload in ENSEMBLE else run_gpu(args)
    if rank == 0 and out is not None:
        if ws == 1 and not args.no_cpu_baseline:
            val, wall = cpu_reference(args.workload, args.cpu_steps, 0, 1, args.advection, grids=1)
            out["cpu_baseline"] = {"value": val, "unit": "cell-steps/s", "cores": 1, "kind": "port",
                                   "sample": f"{args.cpu_steps} steps of {WORKLOADS[args.workload][:3]} on one core "
                                             f"({wall:.1f} s) with the oracle's restatement of the reference step"}
        print(json.dumps(out))


if __name__ == "__main__":
    main()
