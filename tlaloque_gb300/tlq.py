"""ctypes binding of libtlq (the C ABI in include/tlq.h).

This is the Python face of the drop-in: the same entry points a Fortran host
binds through ISO_C_BINDING.  Host arrays are numpy float64 arrays in the
reference layout ``A(1:5, -1:nx+2, -1:ny+2, -1:nz+2)`` (Fortran order).
There is no CPU fallback: without the built library every call fails.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libtlq.so")

OK, ERR_CUDA, ERR_CONFIG, ERR_NONFINITE_DT, ERR_NEG_DENSITY, ERR_TIMEOUT, ERR_ARG, ERR_STATE, ERR_NOMEM = range(9)
BC_OUTFLOW, BC_REFLECTIVE, BC_PERIODIC, BC_INFLOW = 1, 2, 3, 4
LIMITER_NONE, LIMITER_VANLEER, LIMITER_MINMOD, LIMITER_UMIST, LIMITER_WOODWARD, LIMITER_SUPERBEE = 1, 2, 3, 4, 5, 6
SOLVER_HLLC, SOLVER_HLL = 0, 1
COOL_NONE, COOL_REF, COOL_SUBCYCLE, COOL_MLP, COOL_EXACT = 0, 1, 2, 3, 4
MLP_NPARAM = 8641
PREC_FP64, PREC_MIXED = 0, 1
GBC_ZERO, GBC_MULTIPOLE = 0, 1
OUT_DAT, OUT_VTK, OUT_BIN = 1, 2, 3

# Every function the header declares (checked by the CPU test suite).
EXPORTS = (
    "tlq_config_default", "tlq_create", "tlq_destroy", "tlq_set_stream", "tlq_set_cooling_table", "tlq_set_winds",
    "tlq_set_point_masses", "tlq_upload", "tlq_download", "tlq_set_time", "tlq_get_time", "tlq_step", "tlq_advance",
    "tlq_run_until", "tlq_synchronize", "tlq_stats_get", "tlq_enable_timing", "tlq_last_error", "tlq_status_string",
    "tlq_conserved_sums", "tlq_calc_prims", "tlq_time_step", "tlq_fluxes", "tlq_godunov", "tlq_borders",
    "tlq_viscous_step", "tlq_cooling", "tlq_point_potential", "tlq_gravity_source", "tlq_multigrid",
    "tlq_time_step_noalloc", "tlq_measure_fp64_rate",
    "tlq_surrogate_opts_default", "tlq_train_cooling_surrogate", "tlq_get_cooling_surrogate",
    "tlq_set_cooling_surrogate", "tlq_cooling_pairs", "tlq_mlp_loss_grad", "tlq_mlp_infer",
    "tlq_set_tfin", "tlq_set_plane_winds", "tlq_output", "tlq_output_wait", "tlq_set_tiling", "tlq_get_tiling", "tlq_autotune", "tlq_batch_create", "tlq_batch_destroy", "tlq_batch_size", "tlq_batch_member",
    "tlq_batch_set_tiling", "tlq_batch_get_tiling", "tlq_batch_autotune", "tlq_batch_run", "tlq_batch_synchronize",
    "tlq_batch_status", "tlq_batch_enable_timing", "tlq_batch_stats_get", "tlq_batch_last_error",
)


class TlqError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"tlq error {code}: {msg}")
        self.code = code


class CConfig(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("xl", C.c_double), ("xr", C.c_double), ("yl", C.c_double), ("yr", C.c_double),
        ("zl", C.c_double), ("zr", C.c_double),
        ("gamma", C.c_double), ("cfl", C.c_double), ("eta", C.c_double), ("mu0", C.c_double),
        ("cooling_limit", C.c_double),
        ("limiter", C.c_int), ("solver", C.c_int), ("bc", C.c_int * 6), ("cooling", C.c_int),
        ("cool_max_sub", C.c_int), ("cool_sub_frac", C.c_double), ("precision", C.c_int), ("device", C.c_int),
        ("cool_mlp_tol", C.c_double),
        ("self_gravity", C.c_int), ("grav_bc", C.c_int),
    ]


class CWind(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("xc", "yc", "zc", "vx", "vy", "vz", "radius", "mdot", "vinf", "temp", "mu")]


class CPlaneWind(C.Structure):
    _fields_ = [("plane", C.c_int), ("rho", C.c_double), ("vel", C.c_double), ("temp", C.c_double),
                ("mu", C.c_double)]


class CStats(C.Structure):
    _fields_ = [
        ("steps", C.c_longlong), ("t", C.c_double), ("dt", C.c_double), ("status", C.c_int), ("graph", C.c_int),
        ("ms_stage1", C.c_double), ("ms_stage2", C.c_double), ("timed", C.c_longlong), ("bytes_state", C.c_double),
        ("cool_mlp", C.c_longlong), ("cool_fallback", C.c_longlong), ("ms_cool", C.c_double),
        ("cool_single", C.c_longlong), ("ms_grav", C.c_double),
    ]


class CBatchStats(C.Structure):
    _fields_ = [("members", C.c_int), ("cells", C.c_longlong), ("steps", C.c_longlong),
                ("steps_timed", C.c_longlong), ("ms_per_step", C.c_double), ("items", C.c_int), ("blocks", C.c_int),
                ("launches_per_step", C.c_int), ("graph", C.c_int)]


class CSurrogateOpts(C.Structure):
    _fields_ = [("nsamples", C.c_longlong), ("epochs", C.c_int), ("batch", C.c_int), ("lr", C.c_float),
                ("seed", C.c_ulonglong), ("box", C.c_double * 6), ("sub_frac", C.c_double), ("max_sub", C.c_int)]


class CSurrogateReport(C.Structure):
    _fields_ = [("loss_first", C.c_double), ("loss_last", C.c_double), ("val_rmse_y", C.c_double),
                ("val_max_rel_T", C.c_double), ("val_p99_rel_T", C.c_double), ("val_accept", C.c_double),
                ("ms_generate", C.c_double),
                ("ms_train", C.c_double), ("steps", C.c_longlong)]


_lib = None


def measure_fp64_rate(device: int = 0) -> dict:
    """FP64 pipe throughput of `device` (tlq_measure_fp64_rate): FMA,
    IEEE division and square root operations per second."""
    L = load_library()
    f, d, q = C.c_double(), C.c_double(), C.c_double()
    rc = L.tlq_measure_fp64_rate(device, C.byref(f), C.byref(d), C.byref(q))
    if rc != OK:
        raise TlqError(rc, "measure_fp64_rate")
    return {"fma_per_s": f.value, "div_per_s": d.value, "sqrt_per_s": q.value}


def load_library(path: str = LIB_PATH):
    """Load libtlq.so; raises if it has not been built (no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"libtlq.so is not built ({path}); run __graft_entry__.build()")
    L = C.CDLL(path)
    D = C.POINTER(C.c_double)
    V = C.c_void_p
    I = C.c_int
    sig = {
        "tlq_config_default": (None, [C.POINTER(CConfig)]),
        "tlq_measure_fp64_rate": (I, [I, D, D, D]),
        "tlq_create": (I, [C.POINTER(CConfig), C.POINTER(V)]),
        "tlq_destroy": (I, [V]),
        "tlq_set_tfin": (I, [V, C.c_double]),
        "tlq_set_plane_winds": (I, [V, C.POINTER(CPlaneWind), I]),
        "tlq_output": (I, [V, I, C.c_char_p, I, I]),
        "tlq_output_wait": (I, [V]),
        "tlq_set_tiling": (I, [V, I]),
        "tlq_get_tiling": (I, [V, C.POINTER(I)]),
        "tlq_autotune": (I, [V, C.c_char_p, I, C.POINTER(I)]),
        "tlq_batch_create": (I, [C.POINTER(CConfig), I, C.POINTER(V)]),
        "tlq_batch_destroy": (I, [V]),
        "tlq_batch_size": (I, [V]),
        "tlq_batch_member": (V, [V, I]),
        "tlq_batch_set_tiling": (I, [V, I, I]),
        "tlq_batch_get_tiling": (I, [V, I, C.POINTER(I)]),
        "tlq_batch_autotune": (I, [V, C.c_char_p, I, C.POINTER(I)]),
        "tlq_batch_run": (I, [V, I]),
        "tlq_batch_synchronize": (I, [V]),
        "tlq_batch_status": (I, [V, C.POINTER(I)]),
        "tlq_batch_enable_timing": (I, [V, I]),
        "tlq_batch_stats_get": (I, [V, C.POINTER(CBatchStats)]),
        "tlq_batch_last_error": (C.c_char_p, [V]),
        "tlq_set_stream": (I, [V, V]),
        "tlq_set_cooling_table": (I, [V, D, D, I]),
        "tlq_set_winds": (I, [V, C.POINTER(CWind), I]),
        "tlq_set_point_masses": (I, [V, D, I]),
        "tlq_upload": (I, [V, D]),
        "tlq_download": (I, [V, D, D]),
        "tlq_set_time": (I, [V, C.c_double, I]),
        "tlq_get_time": (I, [V, D, C.POINTER(I), D]),
        "tlq_step": (I, [V, D, C.POINTER(I), D]),
        "tlq_advance": (I, [V, I]),
        "tlq_run_until": (I, [V, C.c_double, I, D, C.POINTER(I), D]),
        "tlq_synchronize": (I, [V]),
        "tlq_stats_get": (I, [V, C.POINTER(CStats)]),
        "tlq_enable_timing": (I, [V, I]),
        "tlq_last_error": (C.c_char_p, [V]),
        "tlq_status_string": (C.c_char_p, [I]),
        "tlq_conserved_sums": (I, [V, D]),
        "tlq_calc_prims": (I, [V, D, D]),
        "tlq_time_step": (I, [V, D, D]),
        "tlq_fluxes": (I, [V, D, D, D, D, D, I]),
        "tlq_godunov": (I, [V, D, D, D, D, D, D, C.c_double]),
        "tlq_borders": (I, [V, D, I]),
        "tlq_viscous_step": (I, [V, D, D, D, C.POINTER(I), C.c_double]),
        "tlq_cooling": (I, [V, D, D, C.c_double]),
        "tlq_point_potential": (I, [V, D]),
        "tlq_gravity_source": (I, [V, D, D, D]),
        "tlq_multigrid": (I, [V, D, D, I, C.POINTER(I)]),
        "tlq_time_step_noalloc": (I, [V, I, I, I, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double, V, V]),
        "tlq_surrogate_opts_default": (None, [C.POINTER(CSurrogateOpts)]),
        "tlq_train_cooling_surrogate": (I, [V, C.POINTER(CSurrogateOpts), C.POINTER(CSurrogateReport)]),
        "tlq_get_cooling_surrogate": (I, [V, C.POINTER(C.c_float), C.POINTER(C.c_float), D]),
        "tlq_set_cooling_surrogate": (I, [V, C.POINTER(C.c_float), C.POINTER(C.c_float), D]),
        "tlq_cooling_pairs": (I, [V, C.c_longlong, C.c_ulonglong, D, C.c_double, I, C.POINTER(C.c_float),
                                  C.POINTER(C.c_float), D]),
        "tlq_mlp_loss_grad": (I, [C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float),
                                  C.POINTER(C.c_float), I, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
        "tlq_mlp_infer": (I, [C.POINTER(C.c_float), C.POINTER(C.c_float), I, C.POINTER(C.c_float)]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def _dp(a):
    if a is None:
        return None
    if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and (a.flags.f_contiguous or a.flags.c_contiguous)):
        raise TypeError("expected a contiguous float64 numpy array")
    return a.ctypes.data_as(C.POINTER(C.c_double))


@dataclass
class Wind:
    """tlq_wind / spherical_wind_type (source/winds.f90:5-16)."""
    xc: float = 0.0
    yc: float = 0.0
    zc: float = 0.0
    vx: float = 0.0
    vy: float = 0.0
    vz: float = 0.0
    radius: float = 0.0
    mdot: float = 0.0
    vinf: float = 0.0
    temp: float = 1.0e4
    mu: float = 1.0


@dataclass
class PlaneWind:
    """tlq_plane_wind / plane_wind_type (source/winds.f90:15-28)."""
    plane: int = 1
    rho: float = 1.0
    vel: float = 0.0
    temp: float = 1.0e4
    mu: float = 1.0


@dataclass
class Config:
    """tlq_config: the runtime image of user/parameters.f90 (its defaults)."""
    nx: int = 50
    ny: int = 50
    nz: int = 50
    xl: float = -1.0
    xr: float = 1.0
    yl: float = -1.0
    yr: float = 1.0
    zl: float = -1.0
    zr: float = 1.0
    gamma: float = 5.0 / 3.0
    cfl: float = 0.4
    eta: float = 0.5e-2
    mu0: float = 1.0
    cooling_limit: float = 0.5
    limiter: int = LIMITER_VANLEER
    solver: int = SOLVER_HLLC
    bc: tuple = (BC_REFLECTIVE,) * 6
    cooling: int = COOL_NONE
    cool_max_sub: int = 1
    cool_sub_frac: float = 0.1
    cool_mlp_tol: float = 1e-3
    self_gravity: int = 0  # the reference's -DGRAV MultiGrid; nx = ny = nz = 2^L
    grav_bc: int = GBC_ZERO  # GBC_ZERO (its serial build) or GBC_MULTIPOLE (its MPI build on one rank)
    precision: int = PREC_FP64
    device: int = 0
    # run-time tables (not part of tlq_config; set through their own calls)
    cool_T: np.ndarray | None = None
    cool_logL: np.ndarray | None = None
    winds: list = field(default_factory=list)
    masses: np.ndarray | None = None  # (n, 4): x, y, z, M
    plane_winds: list = field(default_factory=list)

    @property
    def shape(self):
        return (5, self.nx + 4, self.ny + 4, self.nz + 4)

    @property
    def phi_shape(self):
        return (self.nx + 2, self.ny + 2, self.nz + 2)

    @property
    def dx(self):
        return (self.xr - self.xl) / self.nx

    @property
    def dy(self):
        return (self.yr - self.yl) / self.ny

    @property
    def dz(self):
        return (self.zr - self.zl) / self.nz

    @property
    def cells(self) -> int:
        return self.nx * self.ny * self.nz

    def zeros(self) -> np.ndarray:
        return np.zeros(self.shape, dtype=np.float64, order="F")

    def to_c(self) -> CConfig:
        c = CConfig()
        for n in ("nx", "ny", "nz", "limiter", "solver", "cooling", "cool_max_sub", "precision", "device",
                  "self_gravity", "grav_bc"):
            setattr(c, n, int(getattr(self, n)))
        for n in ("xl", "xr", "yl", "yr", "zl", "zr", "gamma", "cfl", "eta", "mu0", "cooling_limit", "cool_sub_frac",
                  "cool_mlp_tol"):
            setattr(c, n, float(getattr(self, n)))
        for q in range(6):
            c.bc[q] = int(self.bc[q])
        return c


class Context:
    """One tlq_ctx: the whole mesh resident on one GPU."""

    def __init__(self, cfg: Config, _borrowed=None):
        self.L = load_library()
        self.cfg = cfg
        self._owned = _borrowed is None
        if _borrowed is None:
            h = C.c_void_p()
            cc = cfg.to_c()
            rc = self.L.tlq_create(C.byref(cc), C.byref(h))
            if rc != OK:
                raise TlqError(rc, f"tlq_create: {self.L.tlq_status_string(rc).decode()}")
        else:
            h = C.c_void_p(_borrowed)
        self.h = h
        if cfg.cool_T is not None:
            T = np.ascontiguousarray(cfg.cool_T, dtype=np.float64)
            Lm = np.ascontiguousarray(cfg.cool_logL, dtype=np.float64)
            self._check(self.L.tlq_set_cooling_table(self.h, _dp(T), _dp(Lm), len(T)), "set_cooling_table")
        if cfg.winds:
            arr = (CWind * len(cfg.winds))()
            for q, w in enumerate(cfg.winds):
                for n, _ in CWind._fields_:
                    setattr(arr[q], n, float(getattr(w, n)))
            self._check(self.L.tlq_set_winds(self.h, arr, len(cfg.winds)), "set_winds")
        if cfg.masses is not None and len(cfg.masses):
            m = np.ascontiguousarray(cfg.masses, dtype=np.float64).reshape(-1, 4)
            self._check(self.L.tlq_set_point_masses(self.h, _dp(m), m.shape[0]), "set_point_masses")
        if cfg.plane_winds:
            arr = (CPlaneWind * len(cfg.plane_winds))()
            for q, w in enumerate(cfg.plane_winds):
                arr[q].plane = int(w.plane)
                for n in ("rho", "vel", "temp", "mu"):
                    setattr(arr[q], n, float(getattr(w, n)))
            self._check(self.L.tlq_set_plane_winds(self.h, arr, len(cfg.plane_winds)), "set_plane_winds")

    # -- plumbing ------------------------------------------------------------
    def _check(self, rc: int, what: str):
        if rc != OK:
            msg = self.L.tlq_last_error(self.h).decode() if self.h else ""
            raise TlqError(rc, f"{what}: {self.L.tlq_status_string(rc).decode()} {msg}")

    def close(self):
        if getattr(self, "h", None):
            if getattr(self, "_owned", True):
                self.L.tlq_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- run -----------------------------------------------------------------
    def set_stream(self, stream_handle: int | None):
        self._check(self.L.tlq_set_stream(self.h, C.c_void_p(stream_handle or 0)), "set_stream")

    def upload(self, U: np.ndarray):
        assert U.shape == self.cfg.shape
        self._check(self.L.tlq_upload(self.h, _dp(U)), "upload")

    def download(self, U: np.ndarray | None = None, W: np.ndarray | None = None):
        self._check(self.L.tlq_download(self.h, _dp(U), _dp(W)), "download")
        return U, W

    def state(self):
        U = self.cfg.zeros()
        W = self.cfg.zeros()
        self.download(U, W)
        return U, W

    def set_time(self, t: float, it: int = 0):
        self._check(self.L.tlq_set_time(self.h, float(t), int(it)), "set_time")

    def time(self):
        t, dt, it = C.c_double(), C.c_double(), C.c_int()
        rc = self.L.tlq_get_time(self.h, C.byref(t), C.byref(it), C.byref(dt))
        return t.value, it.value, dt.value, rc

    def step(self, check: bool = True):
        t, dt, it = C.c_double(), C.c_double(), C.c_int()
        rc = self.L.tlq_step(self.h, C.byref(t), C.byref(it), C.byref(dt))
        if check:
            self._check(rc, "step")
        return t.value, it.value, dt.value

    def advance(self, n: int):
        self._check(self.L.tlq_advance(self.h, int(n)), "advance")

    def run_until(self, tfin: float, max_steps: int = 1 << 30):
        t, dt, it = C.c_double(), C.c_double(), C.c_int()
        self._check(self.L.tlq_run_until(self.h, float(tfin), int(max_steps), C.byref(t), C.byref(it), C.byref(dt)),
                    "run_until")
        return t.value, it.value, dt.value

    def output(self, fmt: int, outputpath: str, nout: int, rank: int = 0):
        """Asynchronous output of UPrim in the reference's format (OUT_BIN,
        OUT_DAT, OUT_VTK); returns at once, output_wait() waits."""
        self._check(self.L.tlq_output(self.h, int(fmt), outputpath.encode(), int(nout), int(rank)), "output")

    def output_wait(self):
        self._check(self.L.tlq_output_wait(self.h), "output_wait")

    def set_tiling(self, zlen: int):
        self._check(self.L.tlq_set_tiling(self.h, int(zlen)), "set_tiling")

    def tiling(self) -> int:
        z = C.c_int()
        self._check(self.L.tlq_get_tiling(self.h, C.byref(z)), "get_tiling")
        return z.value

    def autotune(self, cache_path: str | None = None, steps: int = 3) -> int:
        z = C.c_int()
        self._check(self.L.tlq_autotune(self.h, cache_path.encode() if cache_path else None, int(steps), C.byref(z)),
                    "autotune")
        return z.value

    def set_tfin(self, tfin: float):
        self._check(self.L.tlq_set_tfin(self.h, float(tfin)), "set_tfin")

    def synchronize(self):
        self._check(self.L.tlq_synchronize(self.h), "synchronize")

    def enable_timing(self, on: bool = True):
        self._check(self.L.tlq_enable_timing(self.h, int(bool(on))), "enable_timing")

    def stats(self) -> CStats:
        s = CStats()
        self._check(self.L.tlq_stats_get(self.h, C.byref(s)), "stats")
        return s

    def conserved_sums(self) -> np.ndarray:
        out = np.zeros(5)
        self._check(self.L.tlq_conserved_sums(self.h, _dp(out)), "conserved_sums")
        return out

    # -- per-routine entry points ----------------------------------------------
    def calc_prims(self, U):
        W = self.cfg.zeros()
        self._check(self.L.tlq_calc_prims(self.h, _dp(W), _dp(U)), "calc_prims")
        return W

    def time_step(self, W) -> float:
        dt = C.c_double()
        self._check(self.L.tlq_time_step(self.h, _dp(W), C.byref(dt)), "time_step")
        return dt.value

    def fluxes(self, U, W, choice, F=None, G=None, H=None):
        F = self.cfg.zeros() if F is None else F
        G = self.cfg.zeros() if G is None else G
        H = self.cfg.zeros() if H is None else H
        self._check(self.L.tlq_fluxes(self.h, _dp(U), _dp(F), _dp(G), _dp(H), _dp(W), int(choice)), "fluxes")
        return F, G, H

    def godunov(self, UU, F, G, H, dt, W=None, out=None):
        out = self.cfg.zeros() if out is None else out
        self._check(self.L.tlq_godunov(self.h, _dp(out), _dp(UU), _dp(F), _dp(G), _dp(H), _dp(W), float(dt)), "godunov")
        return out

    def borders(self, U, order):
        self._check(self.L.tlq_borders(self.h, _dp(U), int(order)), "borders")
        return U

    def viscous_step(self, U, UP, t, it, dt):
        tt, ii = C.c_double(t), C.c_int(it)
        self._check(self.L.tlq_viscous_step(self.h, _dp(U), _dp(UP), C.byref(tt), C.byref(ii), float(dt)),
                    "viscous_step")
        return tt.value, ii.value

    def cooling(self, W, U, dt):
        self._check(self.L.tlq_cooling(self.h, _dp(W), _dp(U), float(dt)), "cooling")

    def point_potential(self, phi=None):
        phi = np.zeros(self.cfg.phi_shape, order="F") if phi is None else phi
        self._check(self.L.tlq_point_potential(self.h, _dp(phi)), "point_potential")
        return phi

    def gravity_source(self, W, phi):
        S = self.cfg.zeros()
        self._check(self.L.tlq_gravity_source(self.h, _dp(W), _dp(phi), _dp(S)), "gravity_source")
        return S

    def multigrid(self, U, phi, it: int) -> int:
        """One MultiGrid call on U's density; phi ((n+2)^3, Fortran order) is
        updated in place.  Returns the V-cycles run."""
        cyc = C.c_int(0)
        self._check(self.L.tlq_multigrid(self.h, _dp(U), _dp(phi), int(it), C.byref(cyc)), "multigrid")
        return cyc.value

    # -- learned cooling surrogate (TLQ_COOL_MLP) -----------------------------
    def train_cooling_surrogate(self, **opts) -> dict:
        """Generate pairs with the exact integrator, train the network on the
        GPU and install it in this context; returns the training report."""
        o = surrogate_opts(**opts)
        rep = CSurrogateReport()
        self._check(self.L.tlq_train_cooling_surrogate(self.h, C.byref(o), C.byref(rep)), "train_cooling_surrogate")
        return {n: getattr(rep, n) for n, _ in CSurrogateReport._fields_}

    def get_cooling_surrogate(self):
        P = np.zeros(MLP_NPARAM, dtype=np.float32)
        norm = np.zeros(6, dtype=np.float32)
        box = np.zeros(6, dtype=np.float64)
        self._check(self.L.tlq_get_cooling_surrogate(self.h, _fp(P), _fp(norm), _dp(box)), "get_cooling_surrogate")
        return P, norm, box

    def set_cooling_surrogate(self, params, norm, box):
        P = np.ascontiguousarray(params, dtype=np.float32)
        nm = np.ascontiguousarray(norm, dtype=np.float32)
        bx = np.ascontiguousarray(box, dtype=np.float64)
        assert P.size == MLP_NPARAM and nm.size == 6 and bx.size == 6
        self._check(self.L.tlq_set_cooling_surrogate(self.h, _fp(P), _fp(nm), _dp(bx)), "set_cooling_surrogate")

    def cooling_pairs(self, n: int, seed: int, box, sub_frac: float = 0.0, max_sub: int = 20000):
        """(X raw features [n,3], Y targets [n], raw (n, T, T_new, dt) [n,4])
        on the GPU: from the exact integrator's closed form (sub_frac 0) or
        from the sub-cycled integrator with sub-steps of sub_frac and
        sub_frac/2, extrapolated."""
        X = np.zeros((n, 3), dtype=np.float32)
        Y = np.zeros(n, dtype=np.float32)
        R = np.zeros((n, 4), dtype=np.float64)
        bx = np.ascontiguousarray(box, dtype=np.float64)
        self._check(self.L.tlq_cooling_pairs(self.h, int(n), int(seed), _dp(bx), float(sub_frac), int(max_sub),
                                             _fp(X), _fp(Y), _dp(R)), "cooling_pairs")
        return X, Y, R


def _fp(a):
    if not (isinstance(a, np.ndarray) and a.dtype == np.float32 and a.flags.c_contiguous):
        raise TypeError("expected a C-contiguous float32 numpy array")
    return a.ctypes.data_as(C.POINTER(C.c_float))


def surrogate_opts(**kw) -> CSurrogateOpts:
    """tlq_surrogate_opts with the library defaults, overridden by keywords."""
    L = load_library()
    o = CSurrogateOpts()
    L.tlq_surrogate_opts_default(C.byref(o))
    for k, v in kw.items():
        if k == "box":
            for q in range(6):
                o.box[q] = float(v[q])
        else:
            setattr(o, k, v)
    return o


def mlp_loss_grad(params, X, Y, wt=None):
    """Weighted mean squared error of y and its gradient (GPU training kernel)."""
    L = load_library()
    P = np.ascontiguousarray(params, dtype=np.float32)
    Xc = np.ascontiguousarray(X, dtype=np.float32)
    Yc = np.ascontiguousarray(Y, dtype=np.float32)
    Wc = None if wt is None else np.ascontiguousarray(wt, dtype=np.float32)
    g = np.zeros(MLP_NPARAM, dtype=np.float32)
    loss = np.zeros(1, dtype=np.float32)
    rc = L.tlq_mlp_loss_grad(_fp(P), _fp(Xc), _fp(Yc), None if Wc is None else _fp(Wc), int(Yc.size), _fp(g),
                             _fp(loss))
    if rc != OK:
        raise TlqError(rc, f"tlq_mlp_loss_grad: {L.tlq_status_string(rc).decode()}")
    return float(loss[0]), g


def mlp_infer(params, X):
    """Network output y for normalised features X [n,3] (GPU inference kernel)."""
    L = load_library()
    P = np.ascontiguousarray(params, dtype=np.float32)
    Xc = np.ascontiguousarray(X, dtype=np.float32)
    Y = np.zeros(Xc.shape[0], dtype=np.float32)
    rc = L.tlq_mlp_infer(_fp(P), _fp(Xc), int(Xc.shape[0]), _fp(Y))
    if rc != OK:
        raise TlqError(rc, f"tlq_mlp_infer: {L.tlq_status_string(rc).decode()}")
    return Y


class Batch:
    """A tlq_batch: independent meshes advanced together by persistent
    launches over all members' tiles, one CUDA graph per step.  members[i]
    is a Context on member i (set-up, upload, download, time)."""

    def __init__(self, cfgs):
        self.L = load_library()
        arr = (CConfig * len(cfgs))()
        for q, c in enumerate(cfgs):
            arr[q] = c.to_c()
        h = C.c_void_p()
        rc = self.L.tlq_batch_create(arr, len(cfgs), C.byref(h))
        if rc != OK:
            raise TlqError(rc, f"tlq_batch_create: {self.L.tlq_status_string(rc).decode()}")
        self.h = h
        self.members = [Context(c, _borrowed=self.L.tlq_batch_member(h, q)) for q, c in enumerate(cfgs)]

    def _check(self, rc: int, what: str):
        if rc != OK:
            raise TlqError(rc, f"{what}: {self.L.tlq_status_string(rc).decode()} "
                               f"{self.L.tlq_batch_last_error(self.h).decode()}")

    def close(self):
        if getattr(self, "h", None):
            for m in self.members:
                m.h = None
            self.L.tlq_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def run(self, steps: int):
        self._check(self.L.tlq_batch_run(self.h, int(steps)), "batch_run")

    def synchronize(self):
        self._check(self.L.tlq_batch_synchronize(self.h), "batch_synchronize")

    def status(self):
        st = (C.c_int * len(self.members))()
        self._check(self.L.tlq_batch_status(self.h, st), "batch_status")
        return list(st)

    def set_tiling(self, i: int, zlen: int):
        self._check(self.L.tlq_batch_set_tiling(self.h, int(i), int(zlen)), "batch_set_tiling")

    def tiling(self):
        out = []
        for q in range(len(self.members)):
            z = C.c_int()
            self._check(self.L.tlq_batch_get_tiling(self.h, q, C.byref(z)), "batch_get_tiling")
            out.append(z.value)
        return out

    def autotune(self, cache_path: str | None = None, steps: int = 3):
        ch = (C.c_int * len(self.members))()
        self._check(self.L.tlq_batch_autotune(self.h, cache_path.encode() if cache_path else None, int(steps), ch),
                    "batch_autotune")
        return list(ch)

    def enable_timing(self, on: bool = True):
        self._check(self.L.tlq_batch_enable_timing(self.h, 1 if on else 0), "batch_enable_timing")

    def stats(self) -> CBatchStats:
        s = CBatchStats()
        self._check(self.L.tlq_batch_stats_get(self.h, C.byref(s)), "batch_stats")
        return s

