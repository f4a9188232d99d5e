"""ctypes front end of the CPU oracle (test infrastructure only).

The oracle is a scalar FP64 C restatement of tlaloque's hydrodynamic step
(``tlq_oracle.c``).  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` use this module, and only as the checker; the
product path (``tlaloque_gb300``) never imports it.

Arrays are numpy float64 arrays in the reference layout
``A(1:5, -1:nx+2, -1:ny+2, -1:nz+2)`` (Fortran order); numpy index
``[e, i+1, j+1, k+1]`` is Fortran ``A(e+1, i, j, k)``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libtlq_oracle.so")

BC_OUTFLOW, BC_REFLECTIVE, BC_PERIODIC, BC_INFLOW = 1, 2, 3, 4
LIM_NONE, LIM_VANLEER, LIM_MINMOD, LIM_UMIST, LIM_WOODWARD, LIM_SUPERBEE = 1, 2, 3, 4, 5, 6
SOLVER_HLLC, SOLVER_HLL = 0, 1
COOL_NONE, COOL_REF, COOL_SUBCYCLE, COOL_EXACT = 0, 1, 2, 4
GBC_ZERO, GBC_MULTIPOLE = 0, 1


class _Wind(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("xc", "yc", "zc", "vx", "vy", "vz", "radius", "mdot", "vinf", "temp", "mu")]


class _PlaneWind(C.Structure):
    _fields_ = [("plane", C.c_int), ("rho", C.c_double), ("vel", C.c_double), ("temp", C.c_double),
                ("mu", C.c_double)]


class _Params(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("xl", C.c_double), ("xr", C.c_double), ("yl", C.c_double), ("yr", C.c_double),
        ("zl", C.c_double), ("zr", C.c_double),
        ("gamma", C.c_double), ("cfl", C.c_double), ("eta", C.c_double), ("mu0", C.c_double),
        ("cooling_limit", C.c_double),
        ("limiter", C.c_int), ("solver", C.c_int), ("bc", C.c_int * 6), ("cooling", C.c_int),
        ("ncool", C.c_int), ("coolT", C.POINTER(C.c_double)), ("coolC", C.POINTER(C.c_double)),
        ("cool_max_sub", C.c_int), ("cool_sub_frac", C.c_double),
        ("nwinds", C.c_int), ("winds", C.POINTER(_Wind)),
        ("nmasses", C.c_int), ("masses", C.POINTER(C.c_double)),
        ("nthreads", C.c_int),
        ("nplanes", C.c_int), ("planes", C.POINTER(_PlaneWind)),
        ("self_gravity", C.c_int), ("grav_bc", C.c_int),
    ]


class _State(C.Structure):
    _fields_ = [(n, C.POINTER(C.c_double)) for n in ("U", "UP", "UPP", "UPrim", "F", "G", "H", "S", "PHI")] + [
        ("t", C.c_double), ("dt", C.c_double), ("it", C.c_int)] + [
        (n, C.POINTER(C.c_double)) for n in ("PHIG", "PHIT", "MGW")]


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc, no GPU needed)."""
    src = os.path.join(HERE, "tlq_oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        P = C.POINTER(_Params)
        D = C.POINTER(C.c_double)
        L.tlqo_array_len.restype = C.c_long
        L.tlqo_array_len.argtypes = [P]
        L.tlqo_phi_len.restype = C.c_long
        L.tlqo_phi_len.argtypes = [P]
        L.tlqo_calc_prims.argtypes = [P, D, D]
        L.tlqo_time_step.restype = C.c_double
        L.tlqo_time_step.argtypes = [P, D]
        L.tlqo_fluxes.argtypes = [P, D, D, D, D, D, C.c_int]
        L.tlqo_godunov.argtypes = [P, D, D, D, D, D, C.c_double, D]
        L.tlqo_borders.argtypes = [P, D, C.c_int]
        L.tlqo_impose_winds.argtypes = [P, D]
        L.tlqo_step.argtypes = [P, D, D, D, D, C.POINTER(C.c_int), C.c_double]
        L.tlqo_cooling.argtypes = [P, D, D, C.c_double]
        L.tlqo_point_potential.argtypes = [P, D]
        L.tlqo_gravity_source.argtypes = [P, D, D, D]
        L.tlqo_cool_coef.restype = C.c_double
        L.tlqo_cool_coef.argtypes = [P, C.c_double]
        L.tlqo_cool_gcum.argtypes = [P, D]
        L.tlqo_cool_exact_T.restype = C.c_double
        L.tlqo_cool_exact_T.argtypes = [P, D, C.c_double, C.c_double, C.c_double]
        L.tlqo_mg_levels.restype = C.c_int
        L.tlqo_mg_levels.argtypes = [P]
        L.tlqo_mg_work_len.restype = C.c_long
        L.tlqo_mg_work_len.argtypes = [P]
        L.tlqo_multigrid.restype = C.c_int
        L.tlqo_multigrid.argtypes = [P, D, D, C.c_int, D]
        L.tlqo_init.argtypes = [P, C.POINTER(_State)]
        L.tlqo_run.restype = C.c_int
        L.tlqo_run.argtypes = [P, C.POINTER(_State), C.c_int, C.c_double]
        _lib = L
    return _lib


def _ptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.float64 and (a.flags.f_contiguous or a.ndim == 1 or a.flags.c_contiguous)
    return a.ctypes.data_as(C.POINTER(C.c_double))


@dataclass
class Wind:
    """spherical_wind_type (source/winds.f90:5-16)."""
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
class Params:
    """Runtime image of user/parameters.f90 (defaults are that file's)."""
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
    limiter: int = LIM_VANLEER
    solver: int = SOLVER_HLLC
    bc: tuple = (BC_REFLECTIVE,) * 6
    cooling: int = COOL_NONE
    cool_T: np.ndarray | None = None
    cool_logL: np.ndarray | None = None
    cool_max_sub: int = 1
    cool_sub_frac: float = 0.1
    winds: list = field(default_factory=list)
    masses: np.ndarray | None = None  # (n, 4): x, y, z, M
    nthreads: int = 0
    plane_winds: list = field(default_factory=list)  # objects with plane, rho, vel, temp, mu
    self_gravity: int = 0  # MultiGrid self-gravity (the reference's -DGRAV); nx = ny = nz = 2^L
    grav_bc: int = GBC_ZERO

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

    def zeros(self) -> np.ndarray:
        return np.zeros(self.shape, dtype=np.float64, order="F")

    def c_struct(self):
        """Build the C parameter struct; returns (struct, keepalive)."""
        s = _Params()
        keep = []
        for n in ("nx", "ny", "nz", "limiter", "solver", "cooling", "cool_max_sub", "nthreads", "self_gravity",
                  "grav_bc"):
            setattr(s, n, int(getattr(self, n)))
        for n in ("xl", "xr", "yl", "yr", "zl", "zr", "gamma", "cfl", "eta", "mu0", "cooling_limit", "cool_sub_frac"):
            setattr(s, n, float(getattr(self, n)))
        for q in range(6):
            s.bc[q] = int(self.bc[q])
        if self.cool_T is not None:
            T = np.ascontiguousarray(self.cool_T, dtype=np.float64)
            L = np.ascontiguousarray(self.cool_logL, dtype=np.float64)
            keep += [T, L]
            s.ncool, s.coolT, s.coolC = len(T), _ptr(T), _ptr(L)
        if self.winds:
            arr = (_Wind * len(self.winds))()
            for q, w in enumerate(self.winds):
                for n, _ in _Wind._fields_:
                    setattr(arr[q], n, float(getattr(w, n)))
            keep.append(arr)
            s.nwinds, s.winds = len(self.winds), C.cast(arr, C.POINTER(_Wind))
        if self.masses is not None and len(self.masses):
            m = np.ascontiguousarray(self.masses, dtype=np.float64).reshape(-1, 4)
            keep.append(m)
            s.nmasses, s.masses = m.shape[0], _ptr(m)
        if self.plane_winds:
            arr = (_PlaneWind * len(self.plane_winds))()
            for q, w in enumerate(self.plane_winds):
                arr[q].plane = int(w.plane)
                for n in ("rho", "vel", "temp", "mu"):
                    setattr(arr[q], n, float(getattr(w, n)))
            keep.append(arr)
            s.nplanes, s.planes = len(self.plane_winds), C.cast(arr, C.POINTER(_PlaneWind))
        return s, keep


def params_from_config(cfg, nthreads: int = 0) -> Params:
    """The oracle's parameters for a run described by a package ``Config``
    (read by attribute, so the oracle imports nothing of the package)."""
    p = Params(nx=cfg.nx, ny=cfg.ny, nz=cfg.nz, xl=cfg.xl, xr=cfg.xr, yl=cfg.yl, yr=cfg.yr, zl=cfg.zl, zr=cfg.zr,
               gamma=cfg.gamma, cfl=cfg.cfl, eta=cfg.eta, mu0=cfg.mu0, cooling_limit=cfg.cooling_limit,
               limiter=cfg.limiter, solver=cfg.solver, bc=tuple(cfg.bc), cooling=cfg.cooling,
               cool_T=cfg.cool_T, cool_logL=cfg.cool_logL, cool_max_sub=cfg.cool_max_sub,
               cool_sub_frac=cfg.cool_sub_frac, nthreads=nthreads)
    p.winds = [Wind(**{k: getattr(w, k) for k in ("xc", "yc", "zc", "vx", "vy", "vz", "radius", "mdot", "vinf",
                                                   "temp", "mu")}) for w in cfg.winds]
    p.masses = None if cfg.masses is None else np.asarray(cfg.masses, float)
    p.plane_winds = list(getattr(cfg, "plane_winds", []))
    p.self_gravity = int(getattr(cfg, "self_gravity", 0))
    p.grav_bc = int(getattr(cfg, "grav_bc", 0))
    return p


class Oracle:
    """Per-routine calls and the main loop of the restatement."""

    def __init__(self, params: Params):
        self.p = params
        self._s, self._keep = params.c_struct()
        self._pp = C.byref(self._s)
        self.L = lib()

    # per-routine restatements -------------------------------------------
    def calc_prims(self, U):
        W = self.p.zeros()
        self.L.tlqo_calc_prims(self._pp, _ptr(W), _ptr(U))
        return W

    def time_step(self, W) -> float:
        return self.L.tlqo_time_step(self._pp, _ptr(W))

    def multigrid(self, U, phi, it: int):
        """One MultiGrid call (sources.f90:99-193) on the density of U; phi
        ((n+2)^3, Fortran order) is updated in place.  Returns the V-cycles."""
        work = np.zeros(self.L.tlqo_mg_work_len(self._pp), dtype=np.float64)
        assert work.size > 0, "self-gravity needs nx = ny = nz = 2^L"
        return self.L.tlqo_multigrid(self._pp, _ptr(U), _ptr(phi), int(it), _ptr(work))

    def fluxes(self, U, W, choice, F=None, G=None, H=None):
        F = self.p.zeros() if F is None else F
        G = self.p.zeros() if G is None else G
        H = self.p.zeros() if H is None else H
        self.L.tlqo_fluxes(self._pp, _ptr(U), _ptr(F), _ptr(G), _ptr(H), _ptr(W), int(choice))
        return F, G, H

    def godunov(self, UU, F, G, H, dt, S=None, out=None):
        out = self.p.zeros() if out is None else out
        self.L.tlqo_godunov(self._pp, _ptr(out), _ptr(UU), _ptr(F), _ptr(G), _ptr(H), float(dt), _ptr(S))
        return out

    def borders(self, U, order):
        self.L.tlqo_borders(self._pp, _ptr(U), int(order))
        return U

    def impose_winds(self, U):
        self.L.tlqo_impose_winds(self._pp, _ptr(U))
        return U

    def step(self, U, UP, t, it, dt):
        UPP = self.p.zeros()
        tt = C.c_double(t)
        ii = C.c_int(it)
        self.L.tlqo_step(self._pp, _ptr(U), _ptr(UP), _ptr(UPP), C.byref(tt), C.byref(ii), float(dt))
        return tt.value, ii.value

    def cooling(self, W, U, dt):
        self.L.tlqo_cooling(self._pp, _ptr(W), _ptr(U), float(dt))

    def cool_exact_T(self, T: float, tau: float) -> float:
        """The exact integrator's temperature after a step of cooling number
        tau from T (>= the table's first temperature)."""
        g = np.zeros(self.p.cool_T.size)
        self.L.tlqo_cool_gcum(self._pp, _ptr(g))
        return self.L.tlqo_cool_exact_T(self._pp, _ptr(g), float(T), self.cool_coef(T), float(tau))

    def cool_coef(self, T: float) -> float:
        return self.L.tlqo_cool_coef(self._pp, float(T))

    def point_potential(self):
        phi = np.zeros(self.p.phi_shape, dtype=np.float64, order="F")
        self.L.tlqo_point_potential(self._pp, _ptr(phi))
        return phi

    def gravity_source(self, W, phi):
        S = self.p.zeros()
        self.L.tlqo_gravity_source(self._pp, _ptr(W), _ptr(phi), _ptr(S))
        return S


class Run:
    """The main loop of source/mainHD.f90 on the restatement."""

    def __init__(self, params: Params, U0: np.ndarray, _lib=None):
        self.o = Oracle(params)
        if _lib is not None:
            self.o.L = _lib
        p = params
        self.arrays = {n: p.zeros() for n in ("U", "UP", "UPP", "UPrim", "F", "G", "H")}
        self.arrays["U"][...] = U0
        grav = p.masses is not None and len(p.masses) > 0
        if grav or p.self_gravity:
            self.arrays["S"] = p.zeros()
        if grav:
            self.arrays["PHI"] = np.zeros(p.phi_shape, dtype=np.float64, order="F")
        if p.self_gravity:
            self.arrays["PHIG"] = np.zeros(p.phi_shape, dtype=np.float64, order="F")
            self.arrays["PHIT"] = np.zeros(p.phi_shape, dtype=np.float64, order="F")
            self.arrays["MGW"] = np.zeros(self.o.L.tlqo_mg_work_len(self.o._pp), dtype=np.float64)
        st = _State()
        for n in ("U", "UP", "UPP", "UPrim", "F", "G", "H", "S", "PHI", "PHIG", "PHIT", "MGW"):
            setattr(st, n, _ptr(self.arrays.get(n)))
        st.t, st.dt, st.it = 0.0, 0.0, 0
        self.st = st
        self.o.L.tlqo_init(self.o._pp, C.byref(st))

    def run(self, nsteps: int, tfin: float = float("inf")) -> int:
        return self.o.L.tlqo_run(self.o._pp, C.byref(self.st), int(nsteps), float(tfin))

    @property
    def t(self):
        return self.st.t

    @property
    def dt(self):
        return self.st.dt

    @property
    def it(self):
        return self.st.it

    @property
    def U(self):
        return self.arrays["U"]

    @property
    def UPrim(self):
        return self.arrays["UPrim"]


# ---------------------------------------------------------------------------
# FP64 operation counts: the same source compiled with a counting double
# (tlq_oracle_count.cpp); serial, and bit-identical to the oracle.
# ---------------------------------------------------------------------------
COUNT_LIB_PATH = os.path.join(HERE, "_build", "libtlq_oracle_count.so")
_count_lib = None


class _Flops(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("add", "mul", "div", "sqrt", "cmp", "trans")]


def count_lib():
    global _count_lib
    if _count_lib is None:
        srcs = [os.path.join(HERE, f) for f in ("tlq_oracle_count.cpp", "tlq_oracle.c", "tlq_oracle.h")]
        if not os.path.exists(COUNT_LIB_PATH) or os.path.getmtime(COUNT_LIB_PATH) < max(map(os.path.getmtime, srcs)):
            subprocess.run(["make", "-s", "-C", HERE, "count"], check=True)
        L = C.CDLL(COUNT_LIB_PATH)
        L.tlqo_init.argtypes = [C.POINTER(_Params), C.POINTER(_State)]
        L.tlqo_mg_work_len.restype = C.c_long
        L.tlqo_mg_work_len.argtypes = [C.POINTER(_Params)]
        L.tlqo_run.restype = C.c_int
        L.tlqo_run.argtypes = [C.POINTER(_Params), C.POINTER(_State), C.c_int, C.c_double]
        L.tlqo_flops_reset.argtypes = []
        L.tlqo_flops_get.argtypes = [C.POINTER(_Flops)]
        _count_lib = L
    return _count_lib


def count_flops(params: Params, U0: np.ndarray, nsteps: int, tfin: float = float("inf"), skip: int = 0):
    """Run skip uncounted steps, then nsteps counted steps of the main loop on
    the counting build; return (counts per category over the counted steps,
    the Run).  The set-up before the loop (borders, calc_prims, potential) is
    not counted."""
    L = count_lib()
    r = Run(params, U0, _lib=L)  # tlqo_init ran on the counting build
    if skip:
        r.run(skip, tfin)
    L.tlqo_flops_reset()
    n = r.run(nsteps, tfin)
    f = _Flops()
    L.tlqo_flops_get(C.byref(f))
    counts = {k: getattr(f, k) for k, _ in _Flops._fields_}
    counts["steps"] = n
    return counts, r
