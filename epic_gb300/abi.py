"""ctypes mirror of include/epic_gb300.h and numpy-backed storage for its structs.

The structs carry what the reference's timestep() reads from the globals `grid`, `planet`
and `var` (include/epic_datatypes.h:238-627); the arrays keep the reference memory layout
X(k,j,i) = base[i + (j+1)*(ni+2) + k*(ni+2)*(nj+3)] (include/epic.h:407-449).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

EPIC_STEP_PROGS_AND_SYNC_DIAGS = 0
EPIC_SYNC_DIAGS_ONLY = 1
EPIC_UV_AB3 = 0
EPIC_UV_LEAPFROG = 1
EPIC_PREC_FP64 = 0
EPIC_PREC_MIXED = 1
EPIC_PREC_MIXED_FAST = 2
EPIC_ADV_HSU = 0
EPIC_ADV_AKIMA = 1
EPIC_PROFILE_HS_EQ = 0
EPIC_PROFILE_N2 = 1
EPIC_PROFILE_TABLE = 2
EPIC_IO_ALL = 0
EPIC_IO_STATE = 1
EPIC_TURB_OFF = 0
EPIC_TURB_SA_DES = 1
EPIC_DIFFUSION_HORIZONTAL_AND_VERTICAL = 1
EPIC_DIFFUSION_JUST_HORIZONTAL = 2
EPIC_DIFFUSION_JUST_VERTICAL = 3

_dp = C.POINTER(C.c_double)


class EpicGrid(C.Structure):
    _fields_ = [
        ("ni", C.c_int32), ("nj", C.c_int32), ("nk", C.c_int32), ("dt", C.c_int32),
        ("uv_scheme", C.c_int32), ("k_sigma", C.c_int32), ("k_sponge", C.c_int32),
        ("newt_cool_on", C.c_int32), ("newt_cool_adjust", C.c_int32), ("drag_v", C.c_int32),
        ("drag_zonal_avg", C.c_int32), ("jtp", C.c_int32), ("advection_scheme", C.c_int32), ("gas_giant", C.c_int32),
        ("dln", C.c_double), ("dlt", C.c_double), ("dy0", C.c_double),
        ("globe_latbot", C.c_double), ("globe_lattop", C.c_double), ("press0", C.c_double),
        ("topo_scale", C.c_double), ("prandtl", C.c_double), ("tau_drag", C.c_double),
        ("nudiv_nondim", C.c_double),
        ("zeta0", C.c_double), ("zeta1", C.c_double), ("hybrid_alpha", C.c_double),
        ("sigma_sigma", C.c_double),
        ("nu", C.c_double * 9),
        ("re", C.c_double), ("rp", C.c_double), ("cp", C.c_double), ("rgas", C.c_double),
        ("kappa", C.c_double), ("cpr", C.c_double), ("kinvisc", C.c_double), ("lat0", C.c_double), ("hs_kf", C.c_double),
        ("x_h2", C.c_double), ("x_he", C.c_double), ("x_3", C.c_double),
        ("dynvisc", C.c_double), ("turbulence", C.c_int32), ("diffusion_direction", C.c_int32),
        ("stability_factor", C.c_int32), ("pad1", C.c_int32),
        ("lon", _dp), ("lat", _dp), ("rln", _dp), ("rlt", _dp), ("f", _dp), ("m", _dp), ("n", _dp),
        ("mn", _dp), ("g", _dp), ("sigmatheta", _dp), ("dsgth", _dp), ("dsgth_inv", _dp),
        ("h_min", _dp), ("t_sponge_inv", _dp),
    ]


FIELD_NAMES_3D = ["hdry", "theta", "p3", "h3", "p2", "theta2", "t2", "t3", "rho2", "rho3", "exner3",
                  "gz3", "mont3", "heat3", "pv3", "ri2", "div_uv3", "w3", "dzdt3", "u_spinup"]
PROGNOSTIC = ["u", "v", "hdry", "theta"]
# the turbulence closure's arrays (allocated by Fields(turbulence=True) only)
TURB_FIELDS = ["nu_turb", "diffusion_coef_uv", "diffusion_coef_theta", "diffusion_coef_mass"]


class EpicFields(C.Structure):
    _fields_ = ([(n, _dp) for n in ["u", "v", "dudt", "dvdt"]]
                + [(n, _dp) for n in FIELD_NAMES_3D]
                + [("gz_surface", _dp),
                   ("it_zero", C.c_int32), ("it_minus1", C.c_int32), ("it_minus2", C.c_int32),
                   ("pad0", C.c_int32), ("itime", C.c_int64), ("model_time", C.c_int64)]
                + [(n, _dp) for n in TURB_FIELDS])


class EpicHsParams(C.Structure):
    _fields_ = [("ni", C.c_int32), ("nj", C.c_int32), ("nk", C.c_int32), ("dt", C.c_int32),
                ("uv_scheme", C.c_int32), ("advection_scheme", C.c_int32),
                ("ptop", C.c_double), ("pbot", C.c_double), ("p_sigma", C.c_double),
                ("nu_nondim", C.c_double * 9), ("nudiv_nondim", C.c_double), ("lat0", C.c_double),
                ("profile", C.c_int32), ("pad1", C.c_int32), ("n2", C.c_double), ("theta_surface", C.c_double),
                ("t_iso", C.c_double), ("table_p", _dp), ("table_t", _dp), ("table_n", C.c_int32), ("pad2", C.c_int32)]


class EpicJetParams(C.Structure):
    _fields_ = [("njets", C.c_int32), ("pad0", C.c_int32), ("amp_min", C.c_double), ("amp_max", C.c_double),
                ("lat_min", C.c_double), ("lat_max", C.c_double), ("width_min", C.c_double), ("width_max", C.c_double),
                ("vort_frac", C.c_double)]


def _ptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_dp)


@dataclass
class Layout:
    ni: int
    nj: int
    nk: int

    @property
    def shape3(self):
        return (self.nk + 2, self.nj + 3, self.ni + 2)

    @property
    def shape2(self):
        return (self.nj + 3, self.ni + 2)

    @property
    def n3(self):
        return (self.nk + 2) * (self.nj + 3) * (self.ni + 2)

    def interior(self, a3: np.ndarray, kind: str = "h"):
        """View of the cells a field's update loops cover (k rows 1..nk, j per grid, i 1..ni).

        kind 'h': h/u grid j = 0..nj; 'v': v grid j = 1..nj; 'w': interfaces k = 0..nk.
        a3 has shape (..., nk+2, nj+3, ni+2); array index j+1 holds row j.
        """
        if kind == "h":
            return a3[..., 1:self.nk + 1, 1:self.nj + 2, 1:self.ni + 1]
        if kind == "v":
            return a3[..., 1:self.nk + 1, 2:self.nj + 2, 1:self.ni + 1]
        if kind == "uv":   # u, v interfaces the time step updates: k = 1..nk-1
            return a3[..., 1:self.nk, 1:self.nj + 2, 1:self.ni + 1]
        if kind == "vv":
            return a3[..., 1:self.nk, 2:self.nj + 2, 1:self.ni + 1]
        if kind == "w":
            return a3[..., 0:self.nk + 1, 1:self.nj + 2, 1:self.ni + 1]
        raise ValueError(kind)


class GridArrays:
    """Owns the 1-D arrays an EpicGrid points at."""

    def __init__(self, ni: int, nj: int, nk: int, k_sponge: int = 0):
        self.layout = Layout(ni, nj, nk)
        nj1, ni1, nk1 = 2 * (nj + 1) + 1, 2 * (ni + 1) + 1, 2 * (nk + 1) + 1
        self.arrays = {
            "lon": np.zeros(ni1), "lat": np.zeros(nj1), "rln": np.zeros(nj1), "rlt": np.zeros(nj1),
            "f": np.zeros(nj1), "m": np.zeros(nj1), "n": np.zeros(nj1), "mn": np.zeros(nj1),
            "g": np.zeros(nj1), "sigmatheta": np.zeros(nk1), "dsgth": np.zeros(nk1),
            "dsgth_inv": np.zeros(nk1), "h_min": np.zeros(nk + 2), "t_sponge_inv": np.zeros(k_sponge + 1),
        }
        self.p_ref = np.zeros(nk1)
        self.theta_ref = np.zeros(nk1)
        self.struct = EpicGrid()
        for k, a in self.arrays.items():
            setattr(self.struct, k, _ptr(a))

    def __getattr__(self, name):
        arrays = self.__dict__.get("arrays", {})
        if name in arrays:
            return arrays[name]
        raise AttributeError(name)

    def scalars(self) -> dict:
        out = {}
        for name, typ in EpicGrid._fields_:
            if typ is _dp:
                continue
            v = getattr(self.struct, name)
            out[name] = list(v) if name == "nu" else v
        return out


def _pinned_zeros(shape):
    """Page-locked host array (what cudaMemcpyAsync needs to overlap and run at full rate)."""
    import torch
    return torch.zeros(shape, dtype=torch.float64, pin_memory=True).numpy()


class Fields:
    """Owns numpy storage for every EpicFields pointer, in the reference layout.  The 3-D arrays
    are views of one block, back to back in the library's order (u, v, dudt, dvdt, then
    FIELD_NAMES_3D), so that the library moves a whole state with one copy."""

    def __init__(self, ni: int, nj: int, nk: int, uv_scheme: int, pinned: bool = False, turbulence: bool = False):
        self.layout = Layout(ni, nj, nk)
        self.uv_scheme = uv_scheme
        self.turbulence = turbulence
        nvp, ntp = (1, 3) if uv_scheme == EPIC_UV_AB3 else (2, 1)
        s3 = self.layout.shape3
        n3 = int(np.prod(s3))
        zeros = _pinned_zeros if pinned else np.zeros
        planes = [("u", nvp), ("v", nvp), ("dudt", ntp), ("dvdt", ntp)] + [(n, 0) for n in FIELD_NAMES_3D]
        block = zeros((sum(max(q, 1) for _, q in planes) * n3,))
        self.arrays = {}
        off = 0
        for name, q in planes:
            cnt = max(q, 1) * n3
            view = block[off:off + cnt]
            self.arrays[name] = view.reshape(((q,) if q else ()) + s3)
            off += cnt
        self._block = block
        self.arrays["gz_surface"] = zeros(self.layout.shape2)
        if turbulence:
            tb = zeros((len(TURB_FIELDS) * n3,))
            for q, name in enumerate(TURB_FIELDS):
                self.arrays[name] = tb[q * n3:(q + 1) * n3].reshape(s3)
        self.struct = EpicFields()
        for k, a in self.arrays.items():
            setattr(self.struct, k, _ptr(a))
        self.struct.it_zero, self.struct.it_minus1, self.struct.it_minus2 = 0, 1, 2

    def __getattr__(self, name):
        arrays = self.__dict__.get("arrays", {})
        if name in arrays:
            return arrays[name]
        raise AttributeError(name)

    def copy(self, pinned: bool = False) -> "Fields":
        out = Fields(self.layout.ni, self.layout.nj, self.layout.nk, self.uv_scheme, pinned=pinned,
                     turbulence=self.turbulence)
        for k, a in self.arrays.items():
            out.arrays[k][...] = a
        for name in ("it_zero", "it_minus1", "it_minus2", "itime", "model_time"):
            setattr(out.struct, name, getattr(self.struct, name))
        return out

    @property
    def nbytes(self) -> int:
        return int(sum(a.nbytes for a in self.arrays.values()))

    @property
    def state_nbytes(self) -> int:
        """Bytes of the prognostic arrays (u, v, dudt, dvdt, hdry, theta, and nu_turb with the
        turbulence closure): what EPIC_IO_STATE moves."""
        keys = ("u", "v", "dudt", "dvdt", "hdry", "theta") + (("nu_turb",) if self.turbulence else ())
        return int(sum(self.arrays[k].nbytes for k in keys))

    def wind(self, name: str) -> np.ndarray:
        """Current value plane of u or v (grid.it_uv: plane 0 for AB3, IT_ZERO for leapfrog)."""
        a = self.arrays[name]
        return a[0] if self.uv_scheme == EPIC_UV_AB3 else a[self.struct.it_zero]

    def tendency(self, name: str) -> np.ndarray:
        """Most recent tendency plane of u or v."""
        a = self.arrays[name]
        if self.uv_scheme == EPIC_UV_AB3:
            return a[self.struct.it_minus1]   # after the step's index rotation
        return a[0]


@dataclass
class JetConfig:
    """Seeded zonal jets (epic_jet_initial_state): njets Gaussian jets u(lat), constant with
    height, amplitudes, centres and widths uniform in the ranges; a non-divergent perturbation
    with vort_frac of the jets' rms vorticity."""
    njets: int = 6
    amp: tuple = (50.0, 150.0)
    lat: tuple = (-70.0, 70.0)
    width: tuple = (3.0, 8.0)
    vort_frac: float = 0.01

    def params(self) -> EpicJetParams:
        j = EpicJetParams()
        j.njets = self.njets
        j.amp_min, j.amp_max = self.amp
        j.lat_min, j.lat_max = self.lat
        j.width_min, j.width_max = self.width
        j.vort_frac = self.vort_frac
        return j


@dataclass
class HSConfig:
    """A synthetic run on the Held-Suarez planet: grid shape, time step, schemes, dissipation,
    sounding and initial state (state "hs": the sounding's column at rest with theta noise;
    state "jet": the balanced zonal jets of `jet` on the sounding)."""
    ni: int = 64
    nj: int = 32
    nk: int = 10
    dt: int = 300
    uv_scheme: int = EPIC_UV_AB3
    advection_scheme: int = EPIC_ADV_HSU
    nu4: float = 0.5
    nu6: float = 0.0
    nu8: float = 0.0
    nudiv: float = 0.0
    ptop: float = 10.0
    pbot: float = 1.0e5
    p_sigma: float = 900.0e2
    lat0: float = 45.0
    seed: int = 0
    noise_k: float = 0.1
    profile: int = EPIC_PROFILE_HS_EQ
    n2: float = 1.0e-4
    theta_surface: float = 300.0
    t_iso: float = 200.0
    state: str = "hs"
    jet: JetConfig = field(default_factory=JetConfig)
    # EPIC_PROFILE_TABLE: the sounding as (pressures [Pa], temperatures [K]), e.g. the reference's
    # t_vs_p.held_suarez (tests/golden/sounding/t_vs_p_held_suarez.npz)
    table: tuple | None = None
    # the gas-giant lower boundary: GZ_SURFACE from gradient balance with the bottom layer's
    # zonal-mean U in every store_pgrad_vars (planet->type "gas-giant"), instead of the terrain
    gas_giant: bool = False
    # hydrogen thermodynamics (every form): mole fractions of H2 and He; 0 keeps the ideal gas
    x_h2: float = 0.0
    x_he: float = 0.0
    # the Spalart-Allmaras DES turbulence closure (FP64 form): NU_TURB starts at 20 kinvisc
    # everywhere (init_subgrid), the diffusivities at zero; direction and stability factor as
    # grid.diffusion_direction and grid.stability_factor (1 = "Collins et al. (2004)")
    turbulence: bool = False
    diffusion_direction: int = EPIC_DIFFUSION_HORIZONTAL_AND_VERTICAL
    stability_factor: int = 1
    extra: dict = field(default_factory=dict)

    def params(self) -> EpicHsParams:
        p = EpicHsParams()
        p.ni, p.nj, p.nk, p.dt, p.uv_scheme = self.ni, self.nj, self.nk, self.dt, self.uv_scheme
        p.advection_scheme = self.advection_scheme
        p.ptop, p.pbot, p.p_sigma = self.ptop, self.pbot, self.p_sigma
        for i in range(9):
            p.nu_nondim[i] = 0.0
        p.nu_nondim[4], p.nu_nondim[6], p.nu_nondim[8] = self.nu4, self.nu6, self.nu8
        p.nudiv_nondim = self.nudiv
        p.lat0 = self.lat0
        p.profile = self.profile
        p.n2, p.theta_surface, p.t_iso = self.n2, self.theta_surface, self.t_iso
        if self.table is not None:
            # the struct points at these arrays: they live as long as this config
            self._table_arrays = tuple(np.ascontiguousarray(a, dtype=np.float64) for a in self.table)
            tp, tt = self._table_arrays
            if tp.shape != tt.shape:
                raise ValueError("sounding table: pressures and temperatures differ in length")
            p.table_p, p.table_t, p.table_n = _ptr(tp), _ptr(tt), int(tp.size)
        return p

    @property
    def cells(self) -> int:
        return self.ni * self.nj * self.nk
