"""ctypes access to the oracle (test infrastructure only).

Two oracles live under oracle/:
  libepicport.so  the CPU restatement of the reference step (oracle/epic_port.c), built from
                  committed sources anywhere (also on the GPU host);
  libepicport_cr.so  the same restatement with log/exp/pow correctly rounded, the rounding
                  the CUDA kernels use; glibc's pow is not correctly rounded in ~0.1% of calls,
                  so this variant is what the kernels must match bit for bit;
  libepicref.so   the reference's own step compiled from its sources (oracle/Makefile `ref`),
                  only where the reference tree is present.  It keeps static state, so each
                  model runs in a fresh spawned process.
"""
from __future__ import annotations

import ctypes as C
import multiprocessing as mp
import os
import subprocess

import numpy as np

from epic_gb300.abi import EPIC_STEP_PROGS_AND_SYNC_DIAGS, EPIC_SYNC_DIAGS_ONLY, EpicFields, EpicGrid, Fields, GridArrays

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE = os.path.join(ROOT, "oracle")
PORT_LIB = os.path.join(ORACLE, "_build", "libepicport.so")
PORT_CR_LIB = os.path.join(ORACLE, "_build", "libepicport_cr.so")
REF_LIB = os.path.join(ORACLE, "_ref", "libepicref.so")
# where the reference's sources are: oracle/Makefile's REF unless EPIC_REFERENCE_DIR says otherwise
REF_ARGS = [f"REF={os.environ['EPIC_REFERENCE_DIR']}"] if os.environ.get("EPIC_REFERENCE_DIR") else []

_port = {}


def build_port() -> str:
    subprocess.run(["make", "-s", "-C", ORACLE, "port"], check=True)
    return PORT_LIB


def reference_available() -> bool:
    """Whether the reference's sources are present (and its step is built)."""
    if subprocess.run(["make", "-s", "-C", ORACLE, "have-ref", *REF_ARGS], capture_output=True).returncode != 0:
        return False
    r = subprocess.run(["make", "-s", "-j8", "-C", ORACLE, "ref", *REF_ARGS], capture_output=True)
    return r.returncode == 0 and os.path.exists(REF_LIB)


def port_lib(cr_libm: bool = False) -> C.CDLL:
    if cr_libm not in _port:
        build_port()
        lib = C.CDLL(PORT_CR_LIB if cr_libm else PORT_LIB)
        lib.ep_create.restype = C.c_void_p
        lib.ep_create.argtypes = [C.POINTER(EpicGrid)]
        lib.ep_destroy.argtypes = [C.c_void_p]
        lib.ep_destroy.restype = None
        for n in ("ep_upload", "ep_download"):
            getattr(lib, n).argtypes = [C.c_void_p, C.POINTER(EpicFields)]
        for n in ("ep_timestep", "ep_run", "ep_stage"):
            getattr(lib, n).argtypes = [C.c_void_p, C.c_int]
        lib.ep_cfl_dt.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
        lib.ep_error.restype = C.c_char_p
        lib.ep_error.argtypes = [C.c_void_p]
        lib.ep_create_error.restype = C.c_char_p
        _port[cr_libm] = lib
    return _port[cr_libm]


class Port:
    """The CPU restatement of the step on one grid (cr_libm: with correctly rounded log/exp/pow)."""

    def __init__(self, grid: GridArrays, cr_libm: bool = False):
        self.lib = port_lib(cr_libm)
        self.layout = grid.layout
        self.uv_scheme = grid.struct.uv_scheme
        self.turbulence = bool(grid.struct.turbulence)
        h = self.lib.ep_create(C.byref(grid.struct))
        if not h:
            raise RuntimeError("ep_create: " + self.lib.ep_create_error().decode())
        self.h = C.c_void_p(h)

    def _chk(self, rc, what):
        if rc:
            raise RuntimeError(f"{what}: {self.lib.ep_error(self.h).decode()}")

    def upload(self, f: Fields):
        self._chk(self.lib.ep_upload(self.h, C.byref(f.struct)), "ep_upload")

    def download(self) -> Fields:
        f = Fields(self.layout.ni, self.layout.nj, self.layout.nk, self.uv_scheme, turbulence=self.turbulence)
        self._chk(self.lib.ep_download(self.h, C.byref(f.struct)), "ep_download")
        return f

    def timestep(self, action=EPIC_STEP_PROGS_AND_SYNC_DIAGS):
        self._chk(self.lib.ep_timestep(self.h, action), "ep_timestep")

    def run(self, n: int):
        self._chk(self.lib.ep_run(self.h, n), "ep_run")

    def stage(self, s: int):
        self._chk(self.lib.ep_stage(self.h, s), "ep_stage")

    def cfl_dt(self):
        """cfl_dt of the current state: (the int time step, (cflx, cfly, cflz))."""
        c = (C.c_double * 3)()
        dt = self.lib.ep_cfl_dt(self.h, c)
        return int(dt), tuple(c)

    def __del__(self):
        try:
            self.lib.ep_destroy(self.h)
        except Exception:
            pass


def fields_to_dict(f: Fields) -> dict:
    d = {k: v.copy() for k, v in f.arrays.items()}
    for n in ("it_zero", "it_minus1", "it_minus2", "itime", "model_time"):
        d[n] = int(getattr(f.struct, n))
    return d


def dict_to_fields(d: dict, ni, nj, nk, uv_scheme) -> Fields:
    f = Fields(ni, nj, nk, uv_scheme, turbulence="nu_turb" in d)
    for k in f.arrays:
        f.arrays[k][...] = d[k]
    for n in ("it_zero", "it_minus1", "it_minus2", "itime", "model_time"):
        setattr(f.struct, n, int(d[n]))
    return f


def _ref_worker(grid_arrays: dict, grid_scalars: dict, fields: dict, dims, schedule, q):
    """Run the reference harness in this (fresh) process; schedule = [('sync'|'step', n), ...]."""
    try:
        ni, nj, nk, scheme = dims
        ga = GridArrays(ni, nj, nk)
        for k, v in grid_arrays.items():
            ga.arrays[k][...] = v
        for k, v in grid_scalars.items():
            if k == "nu":
                for i in range(9):
                    ga.struct.nu[i] = v[i]
            else:
                setattr(ga.struct, k, v)
        f = dict_to_fields(fields, ni, nj, nk, scheme)
        lib = C.CDLL(REF_LIB)
        rc = lib.ref_init(C.byref(ga.struct), C.byref(f.struct))
        if rc:
            raise RuntimeError(f"ref_init {rc}")
        geo = (C.c_double * 8)()
        lib.ref_geometry_maxdiff(geo)
        out = []
        for what, n in schedule:
            if what == "sync":
                lib.ref_timestep(EPIC_SYNC_DIAGS_ONLY)
            else:
                lib.ref_run(n)
            g = Fields(ni, nj, nk, scheme, turbulence=bool(ga.struct.turbulence))
            lib.ref_get(C.byref(g.struct))
            d = fields_to_dict(g)
            d["cfl_dt"] = int(lib.ref_cfl_dt())
            out.append(d)
        q.put(("ok", list(geo), out))
    except Exception as e:  # pragma: no cover - reported to the parent
        q.put(("err", repr(e), None))


def run_reference(ga: GridArrays, f: Fields, schedule) -> tuple[list, list]:
    """Snapshots of the reference after each schedule entry, computed in a spawned process."""
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    dims = (ga.layout.ni, ga.layout.nj, ga.layout.nk, f.uv_scheme)
    p = ctx.Process(target=_ref_worker, args=({k: v.copy() for k, v in ga.arrays.items()}, ga.scalars(),
                                               fields_to_dict(f), dims, schedule, q))
    p.start()
    import queue
    while True:   # a reference that exits (its epic_error) reports nothing: stop waiting then
        try:
            status, geo, out = q.get(timeout=5)
            break
        except queue.Empty:
            if not p.is_alive():
                raise RuntimeError(f"the reference process ended with exit code {p.exitcode} before reporting")
    p.join(60)
    if status != "ok":
        raise RuntimeError(geo)
    return geo, out


def rel_l2(a: np.ndarray, b: np.ndarray) -> float:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.linalg.norm(b.ravel())
    num = np.linalg.norm((a - b).ravel())
    return float(num / den) if den > 0 else float(num)


def _sounding_worker(pdat, tdat, press0, pres, q):
    try:
        lib = C.CDLL(REF_LIB)
        dp = C.POINTER(C.c_double)
        pdat, tdat, pres = (np.ascontiguousarray(a, dtype=np.float64) for a in (pdat, tdat, pres))
        out = np.zeros(pres.size)
        lib.ref_sounding_theta(C.c_int(pdat.size), pdat.ctypes.data_as(dp), tdat.ctypes.data_as(dp), C.c_double(press0),
                               C.c_int(pres.size), pres.ctypes.data_as(dp), out.ctypes.data_as(dp))
        q.put(("ok", out))
    except Exception as e:  # pragma: no cover - reported to the parent
        q.put(("err", repr(e)))


def reference_sounding_theta(pdat, tdat, press0, pres) -> np.ndarray:
    """theta at `pres` from the reference's own get_sounding on the table (pdat bottom first),
    computed in a spawned process (the reference keeps the table in static storage)."""
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    p = ctx.Process(target=_sounding_worker, args=(np.asarray(pdat), np.asarray(tdat), press0, np.asarray(pres), q))
    p.start()
    status, out = q.get(timeout=600)
    p.join(60)
    if status != "ok":
        raise RuntimeError(out)
    return out
