"""GB300-native drop-in for the EPIC single-processor timestep().

The compute path is the CUDA library epic_gb300/_lib/libepic_gb300.so (C ABI in
include/epic_gb300.h).  This package only loads it and mirrors the reference's calling
interface in Python:

    timestep(planet, action, Buff2D)   src/shared/epic_timestep.c:62   ->  Model.timestep(action)
    the epic driver's step loop        src/shared/epic_main.c:336-427  ->  Model.run(nsteps)
    var_write's need for host data     src/shared/epic_funcs_io.c:1361 ->  Model.download()

There is no CPU fallback: if the library is missing or no GPU is present, Model() raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .abi import (EPIC_ADV_AKIMA, EPIC_ADV_HSU, EPIC_IO_ALL, EPIC_IO_STATE, EPIC_PREC_FP64, EPIC_PREC_MIXED, EPIC_PREC_MIXED_FAST, EPIC_PROFILE_HS_EQ,
                  EPIC_PROFILE_N2, EPIC_PROFILE_TABLE, EPIC_STEP_PROGS_AND_SYNC_DIAGS, EPIC_SYNC_DIAGS_ONLY, EPIC_TURB_OFF,
                  EPIC_TURB_SA_DES, EPIC_UV_AB3, EPIC_UV_LEAPFROG, TURB_FIELDS, EpicFields, EpicGrid, EpicHsParams, EpicJetParams, Fields, GridArrays, HSConfig, JetConfig, Layout)

TUNE_GROUPS = 10   # EPIC_TUNE_GROUPS
TUNE_HSU_MERID_VARIANT = 9   # table entry: 0 automatic, 1 fused march, 2 four passes
_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libepic_gb300.so")
_lib = None


class EpicError(RuntimeError):
    """A C-ABI call returned an error code (the reference would have called epic_error())."""


def load_library(path: str | None = None) -> C.CDLL:
    """Load (once) and return the CUDA library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise EpicError(f"{p} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(p)
    lib.epic_last_error.restype = C.c_char_p
    lib.epic_model_create.argtypes = [C.POINTER(EpicGrid), C.c_int32, C.POINTER(C.c_void_p)]
    lib.epic_model_destroy.argtypes = [C.c_void_p]
    lib.epic_model_destroy.restype = None
    for name in ("epic_model_upload", "epic_model_download"):
        getattr(lib, name).argtypes = [C.c_void_p, C.POINTER(EpicFields)]
    lib.epic_model_timestep.argtypes = [C.c_void_p, C.c_int32]
    lib.epic_model_run.argtypes = [C.c_void_p, C.c_int32]
    lib.epic_model_run_stage.argtypes = [C.c_void_p, C.c_int32]
    lib.epic_model_sync.argtypes = [C.c_void_p]
    lib.epic_model_step_host.argtypes = [C.c_void_p, C.POINTER(EpicFields), C.c_int32, C.c_int32]
    lib.epic_model_stream.argtypes = [C.c_void_p]
    lib.epic_model_stream.restype = C.c_void_p
    lib.epic_model_kernels_per_step.argtypes = [C.c_void_p]
    lib.epic_model_kernels_per_step.restype = C.c_int32
    lib.epic_model_device_bytes.argtypes = [C.c_void_p]
    lib.epic_model_device_bytes.restype = C.c_int64
    lib.epic_model_device.argtypes = [C.c_void_p]
    lib.epic_model_device.restype = C.c_int32
    lib.epic_model_bytes.argtypes = [C.POINTER(EpicGrid), C.c_int32]
    lib.epic_model_bytes.restype = C.c_int64
    lib.epic_model_filter_mass_noalloc.argtypes = [C.c_void_p]
    lib.epic_model_snapshot_begin.argtypes = [C.c_void_p, C.POINTER(EpicFields)]
    lib.epic_model_snapshot_wait.argtypes = [C.c_void_p]
    lib.epic_model_cfl_dt.argtypes = [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_double)]
    lib.epic_batch_create.argtypes = [C.POINTER(C.c_void_p), C.c_int32, C.POINTER(C.c_void_p)]
    lib.epic_batch_destroy.argtypes = [C.c_void_p]
    lib.epic_batch_destroy.restype = None
    for name in ("epic_batch_timestep", "epic_batch_run", "epic_batch_run_stage"):
        getattr(lib, name).argtypes = [C.c_void_p, C.c_int32]
    lib.epic_batch_sync.argtypes = [C.c_void_p]
    lib.epic_batch_query.argtypes = [C.c_void_p]
    lib.epic_batch_stream.argtypes = [C.c_void_p]
    lib.epic_batch_stream.restype = C.c_void_p
    lib.epic_batch_kernels_per_step.argtypes = [C.c_void_p]
    lib.epic_batch_kernels_per_step.restype = C.c_int32
    lib.epic_batch_autotune.argtypes = [C.c_void_p, C.c_int32, C.POINTER(C.c_int32)]
    for name in ("epic_batch_upload", "epic_batch_download"):
        getattr(lib, name).argtypes = [C.c_void_p, C.POINTER(C.POINTER(EpicFields))]
    lib.epic_batch_step_host.argtypes = [C.c_void_p, C.POINTER(C.POINTER(EpicFields)), C.c_int32, C.c_int32, C.c_int32]
    for name in ("epic_batch_set_tuning", "epic_model_set_tuning"):
        getattr(lib, name).argtypes = [C.c_void_p, C.POINTER(C.c_int32)]
    lib.epic_hs_grid_build.argtypes = [C.POINTER(EpicHsParams), C.POINTER(EpicGrid), C.POINTER(C.c_double),
                                       C.POINTER(C.c_double)]
    lib.epic_hs_initial_state.argtypes = [C.POINTER(EpicGrid), C.POINTER(EpicHsParams), C.c_uint64, C.c_double,
                                          C.POINTER(EpicFields)]
    lib.epic_jet_initial_state.argtypes = [C.POINTER(EpicGrid), C.POINTER(EpicHsParams), C.POINTER(EpicJetParams),
                                           C.c_uint64, C.POINTER(EpicFields)]
    _lib = lib
    return lib


def _tuning_table(table: list[int]) -> list[int]:
    table = [int(t) for t in table]
    if len(table) > TUNE_GROUPS:
        raise ValueError(f"a tuning table has at most {TUNE_GROUPS} entries")
    return table + [0] * (TUNE_GROUPS - len(table))


def _check(rc: int, what: str) -> None:
    if rc != 0:
        msg = load_library().epic_last_error().decode(errors="replace")
        raise EpicError(f"{what} failed ({rc}): {msg}")


def hs_setup(cfg: HSConfig) -> tuple[GridArrays, Fields]:
    """Synthetic grid and initial state on the Held-Suarez planet (host only; no GPU needed):
    the sounding's column at rest (cfg.state "hs") or the balanced zonal jets ("jet")."""
    lib = load_library()
    ga = GridArrays(cfg.ni, cfg.nj, cfg.nk)
    p = cfg.params()
    dp = C.POINTER(C.c_double)
    _check(lib.epic_hs_grid_build(C.byref(p), C.byref(ga.struct), ga.p_ref.ctypes.data_as(dp),
                                  ga.theta_ref.ctypes.data_as(dp)), "epic_hs_grid_build")
    ga.struct.gas_giant = int(cfg.gas_giant)
    if cfg.x_h2 > 0.0:   # thermo_setup's cp/R of the mixture (epic_funcs_diag.c:5893-5898), x_3 the rest
        x3 = max(0.0, 1.0 - cfg.x_h2 - cfg.x_he)
        ga.struct.x_h2, ga.struct.x_he, ga.struct.x_3 = cfg.x_h2, cfg.x_he, x3
        ga.struct.cpr = (2.5 * cfg.x_h2 + 2.5 * cfg.x_he + 3.5 * x3) / (cfg.x_h2 + cfg.x_he + x3)
    # planet->dynvisc of the Held-Suarez planet (epic_globals.c:242-253)
    ga.struct.dynvisc = 1.718e-5
    if cfg.turbulence:
        ga.struct.turbulence = EPIC_TURB_SA_DES
        ga.struct.diffusion_direction = cfg.diffusion_direction
        ga.struct.stability_factor = cfg.stability_factor
    f = Fields(cfg.ni, cfg.nj, cfg.nk, cfg.uv_scheme, turbulence=cfg.turbulence)
    if cfg.state == "jet":
        jp = cfg.jet.params()
        _check(lib.epic_jet_initial_state(C.byref(ga.struct), C.byref(p), C.byref(jp), C.c_uint64(cfg.seed),
                                          C.byref(f.struct)), "epic_jet_initial_state")
    elif cfg.state == "hs":
        _check(lib.epic_hs_initial_state(C.byref(ga.struct), C.byref(p), C.c_uint64(cfg.seed), C.c_double(cfg.noise_k),
                                         C.byref(f.struct)), "epic_hs_initial_state")
    else:
        raise ValueError(f"unknown initial state {cfg.state!r}")
    if cfg.turbulence:   # init_subgrid, epic_subgrid.c:2127-2160
        f.nu_turb[...] = ga.struct.kinvisc * 20.0
    return ga, f


def model_bytes(grid: GridArrays, precision: int = EPIC_PREC_FP64) -> int:
    """Device bytes a Model of this grid takes (for admission by memory budget)."""
    return int(load_library().epic_model_bytes(C.byref(grid.struct), precision))


class Model:
    """One device-resident EPIC grid on the current GPU."""

    def __init__(self, grid: GridArrays, precision: int = EPIC_PREC_FP64):
        self.lib = load_library()
        self.grid = grid
        self.layout = grid.layout
        self.uv_scheme = grid.struct.uv_scheme
        self._h = C.c_void_p()
        _check(self.lib.epic_model_create(C.byref(grid.struct), precision, C.byref(self._h)), "epic_model_create")

    def close(self) -> None:
        if self._h:
            self.lib.epic_model_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, f: Fields) -> None:
        _check(self.lib.epic_model_upload(self._h, C.byref(f.struct)), "epic_model_upload")

    def download(self, f: Fields | None = None) -> Fields:
        if f is None:
            f = Fields(self.layout.ni, self.layout.nj, self.layout.nk, self.uv_scheme, turbulence=bool(self.grid.struct.turbulence))
        _check(self.lib.epic_model_download(self._h, C.byref(f.struct)), "epic_model_download")
        return f

    def timestep(self, action: int = EPIC_STEP_PROGS_AND_SYNC_DIAGS) -> None:
        _check(self.lib.epic_model_timestep(self._h, action), "epic_model_timestep")

    def run(self, nsteps: int) -> None:
        _check(self.lib.epic_model_run(self._h, nsteps), "epic_model_run")

    def run_stage(self, stage: int) -> None:
        _check(self.lib.epic_model_run_stage(self._h, stage), "epic_model_run_stage")

    def cfl_dt(self) -> tuple[int, tuple[float, float, float]]:
        """cfl_dt of the device state: (the int time step var_write stores, (cflx, cfly, cflz))."""
        dt = C.c_int32()
        c = (C.c_double * 3)()
        _check(self.lib.epic_model_cfl_dt(self._h, C.byref(dt), c), "epic_model_cfl_dt")
        return int(dt.value), tuple(c)

    def sync(self) -> None:
        _check(self.lib.epic_model_sync(self._h), "epic_model_sync")

    def filter_mass_noalloc(self) -> None:
        """run_stage(10) with the filter's profile tables in the library's fixed device array."""
        _check(self.lib.epic_model_filter_mass_noalloc(self._h), "epic_model_filter_mass_noalloc")

    def snapshot_begin(self, f: Fields) -> None:
        """Start copying the current state into f (pinned) while later steps run; keep f alive."""
        self._snap = f
        _check(self.lib.epic_model_snapshot_begin(self._h, C.byref(f.struct)), "epic_model_snapshot_begin")

    def snapshot_wait(self) -> Fields | None:
        _check(self.lib.epic_model_snapshot_wait(self._h), "epic_model_snapshot_wait")
        f, self._snap = getattr(self, "_snap", None), None
        return f

    def set_tuning(self, table: list[int]) -> None:
        """Launch shapes from Batch.autotune (one entry per kernel group, 0 = built-in; missing
        trailing entries are 0)."""
        arr = (C.c_int32 * TUNE_GROUPS)(*_tuning_table(table))
        _check(self.lib.epic_model_set_tuning(self._h, arr), "epic_model_set_tuning")

    def step_host(self, f: Fields, nsteps: int, prime: bool = False) -> None:
        _check(self.lib.epic_model_step_host(self._h, C.byref(f.struct), int(prime), nsteps), "epic_model_step_host")

    @property
    def stream(self) -> int:
        return self.lib.epic_model_stream(self._h) or 0

    @property
    def kernels_per_step(self) -> int:
        return int(self.lib.epic_model_kernels_per_step(self._h))

    @property
    def device_bytes(self) -> int:
        return int(self.lib.epic_model_device_bytes(self._h))

    @property
    def device(self) -> int:
        """The CUDA device the model was created on."""
        return int(self.lib.epic_model_device(self._h))


class Batch:
    """Several Models of one shape class stepped together: each kernel of the step is launched
    once for all members (epic_batch_* in include/epic_gb300.h).  Upload to and download from
    the member Models; call sync() first."""

    def __init__(self, models: list[Model]):
        self.lib = load_library()
        self.models = list(models)
        arr = (C.c_void_p * len(self.models))(*[m._h.value for m in self.models])
        self._h = C.c_void_p()
        _check(self.lib.epic_batch_create(arr, len(self.models), C.byref(self._h)), "epic_batch_create")

    def close(self) -> None:
        if self._h:
            self.lib.epic_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def timestep(self, action: int = EPIC_STEP_PROGS_AND_SYNC_DIAGS) -> None:
        _check(self.lib.epic_batch_timestep(self._h, action), "epic_batch_timestep")

    def run(self, nsteps: int) -> None:
        _check(self.lib.epic_batch_run(self._h, nsteps), "epic_batch_run")

    def run_stage(self, stage: int) -> None:
        _check(self.lib.epic_batch_run_stage(self._h, stage), "epic_batch_run_stage")

    def _ptrs(self, fields: list[Fields]):
        if len(fields) != len(self.models):
            raise ValueError("one Fields per member")
        return (C.POINTER(EpicFields) * len(fields))(*[C.pointer(f.struct) for f in fields])

    def upload(self, fields: list[Fields]) -> None:
        """Every member's state from host arrays (pinned for full speed), one synchronisation."""
        _check(self.lib.epic_batch_upload(self._h, self._ptrs(fields)), "epic_batch_upload")

    def download(self, fields: list[Fields]) -> list[Fields]:
        _check(self.lib.epic_batch_download(self._h, self._ptrs(fields)), "epic_batch_download")
        return fields

    def step_host(self, fields: list[Fields], nsteps: int = 1, groups: int = 4, io: int = 0) -> list[Fields]:
        """End-to-end steps with host-resident (pinned) state, copies overlapped with kernels.
        io = EPIC_IO_ALL (0) moves every array each way, EPIC_IO_STATE (1) the prognostic arrays
        (u, v, dudt, dvdt, hdry, theta, and nu_turb with the turbulence closure) only and leaves the
        diagnostics on the device."""
        _check(self.lib.epic_batch_step_host(self._h, self._ptrs(fields), groups, nsteps, io), "epic_batch_step_host")
        return fields

    def autotune(self, trial_steps: int = 3) -> list[int]:
        """Pick the block size of each kernel group by timing whole steps (advances the state)."""
        arr = (C.c_int32 * TUNE_GROUPS)()
        _check(self.lib.epic_batch_autotune(self._h, trial_steps, arr), "epic_batch_autotune")
        return list(arr)

    def set_tuning(self, table: list[int]) -> None:
        arr = (C.c_int32 * TUNE_GROUPS)(*_tuning_table(table))
        _check(self.lib.epic_batch_set_tuning(self._h, arr), "epic_batch_set_tuning")

    def sync(self) -> None:
        _check(self.lib.epic_batch_sync(self._h), "epic_batch_sync")

    def done(self) -> bool:
        """True once the work queued on the batch has finished (does not wait; errors of the
        members surface on sync())."""
        rc = self.lib.epic_batch_query(self._h)
        if rc < 0:
            _check(rc, "epic_batch_query")
        return rc == 1

    @property
    def stream(self) -> int:
        return self.lib.epic_batch_stream(self._h) or 0

    @property
    def kernels_per_step(self) -> int:
        return int(self.lib.epic_batch_kernels_per_step(self._h))


__all__ = ["Model", "Batch", "model_bytes", "hs_setup", "load_library", "EpicError", "HSConfig", "Fields", "GridArrays", "Layout",
           "EPIC_ADV_AKIMA", "EPIC_ADV_HSU", "EPIC_PREC_FP64", "EPIC_PREC_MIXED", "EPIC_PREC_MIXED_FAST", "EPIC_STEP_PROGS_AND_SYNC_DIAGS", "EPIC_SYNC_DIAGS_ONLY",
           "EPIC_UV_AB3", "EPIC_UV_LEAPFROG", "EPIC_TURB_OFF", "EPIC_TURB_SA_DES", "TURB_FIELDS", "LIB_PATH", "TUNE_GROUPS", "TUNE_HSU_MERID_VARIANT", "np"]
