"""Problem set-ups: the initial conditions and parameters of each workload.

These play the role of user/user.f90's ``user_initconds`` and of the
parameters.f90 files the reference's test harness generates
(tests_utilities.jl:212-284, :400-547).  Each builder returns a
``(Config, U0)`` pair; U0 is in the reference layout with every cell
(ghosts included) set, as ``user_initconds`` does; the caller then applies
``borders(U, 1)`` (mainHD.f90:38) before uploading.
"""
from __future__ import annotations

import numpy as np

from .tlq import (BC_OUTFLOW, BC_PERIODIC, COOL_SUBCYCLE, GBC_MULTIPOLE, LIMITER_VANLEER, SOLVER_HLL, SOLVER_HLLC,
                  Config, Wind)

# source/constants.f90:6-15 (cgs)
AMU = 1.660538782e-24
KB = 1.380650400e-16
GR = 6.67430e-8
PC = 3.085677588e18
YEAR = 3.155673600e7
MSUN = 1.988920000e33
KMS = 1.0e5
PI_REF = 3.14159265358979


def cell_centres(cfg: Config):
    """x, y, z of every cell index -1..n+2 (HydroCore.f90:35-77)."""
    i = np.arange(-1, cfg.nx + 3, dtype=np.float64)
    j = np.arange(-1, cfg.ny + 3, dtype=np.float64)
    k = np.arange(-1, cfg.nz + 3, dtype=np.float64)
    x = (cfg.xl + cfg.dx * i) - cfg.dx / 2.0
    y = (cfg.yl + cfg.dy * j) - cfg.dy / 2.0
    z = (cfg.zl + cfg.dz * k) - cfg.dz / 2.0
    return x, y, z


def conserved(cfg: Config, rho, vx, vy, vz, p) -> np.ndarray:
    """Primitive fields (broadcastable to the mesh) -> U in the reference layout,
    U(5) = 0.5 rho |v|^2 + p/(gamma-1) as user.f90 writes it."""
    U = cfg.zeros()
    shp = U.shape[1:]
    rho = np.broadcast_to(rho, shp)
    vx, vy, vz, p = (np.broadcast_to(a, shp) for a in (vx, vy, vz, p))
    U[0] = rho
    U[1] = rho * vx
    U[2] = rho * vy
    U[3] = rho * vz
    U[4] = 0.5 * rho * ((vx * vx + vy * vy) + vz * vz) + p / (cfg.gamma - 1.0)
    return U


# ---------------------------------------------------------------------------
def sod_tube(nx: int = 256, solver: int = SOLVER_HLL, eta: float = 0.5e-2):
    """Classic Sod shock tube: 256x4x4 on [0,1] (dy = dz = dx), gamma 1.4,
    (1, 0, 1) | (0.125, 0, 0.1) at x = 0.5, HLL, CFL 0.4, outflow; t = 0.2."""
    dx = 1.0 / nx
    cfg = Config(nx=nx, ny=4, nz=4, xl=0.0, xr=1.0, yl=0.0, yr=4 * dx, zl=0.0, zr=4 * dx, gamma=1.4, cfl=0.4,
                 eta=eta, limiter=LIMITER_VANLEER, solver=solver, bc=(BC_OUTFLOW,) * 6)
    x, _, _ = cell_centres(cfg)
    left = (x < 0.5)[:, None, None]
    rho = np.where(left, 1.0, 0.125)
    p = np.where(left, 1.0, 0.1)
    return cfg, conserved(cfg, rho, 0.0, 0.0, 0.0, p)


SOD_TFIN = 0.2


def sedov(n: int = 128, cfl: float = 0.3, eta: float = 0.5e-2, E0: float = 1.0, rho0: float = 1.0, p0: float = 1e-5):
    """3-D Sedov-Taylor blast: n^3 on [-0.5, 0.5]^3, gamma 5/3, HLLC, outflow,
    CFL 0.3; E0 = 1 spread as thermal energy uniformly over the cells whose
    centre has r < 3 dx (so the deposited energy is E0 exactly); t = 0.05."""
    cfg = Config(nx=n, ny=n, nz=n, xl=-0.5, xr=0.5, yl=-0.5, yr=0.5, zl=-0.5, zr=0.5, gamma=5.0 / 3.0, cfl=cfl,
                 eta=eta, limiter=LIMITER_VANLEER, solver=SOLVER_HLLC, bc=(BC_OUTFLOW,) * 6)
    x, y, z = cell_centres(cfg)
    r = np.sqrt(x[:, None, None] ** 2 + y[None, :, None] ** 2 + z[None, None, :] ** 2)
    inside = r < 3.0 * cfg.dx
    interior = np.zeros_like(inside)
    interior[2:-2, 2:-2, 2:-2] = True
    ncell = int(np.count_nonzero(inside & interior))
    dV = cfg.dx * cfg.dy * cfg.dz
    p_in = (cfg.gamma - 1.0) * E0 / (ncell * dV)
    p = np.where(inside, p_in, p0)
    return cfg, conserved(cfg, rho0, 0.0, 0.0, 0.0, p)


SEDOV_TFIN = 0.05


def sedov_shock_radius(t: float, E0: float = 1.0, rho0: float = 1.0, xi0: float = 1.151666417967) -> float:
    """R_s = xi0 (E t^2 / rho)^(1/5); xi0 for gamma = 5/3 (solutions/sedov_solution_53.txt:3).
    The reference's analysis overlays 1.15 (E t^2/rho)^(1/5) (utils_analisis.jl:1-3)."""
    return xi0 * (E0 * t * t / rho0) ** 0.2


def diagonal_sod(n: int = 150):
    """The reference's own Sod test (tests_utilities.jl:214-224, :402-448): n^3
    on [-0.25, 0.25]^3, gamma 5/3, rho 4, p 1 where -x-y-z > 0, else rho 1,
    p 0.1795; CFL 0.8, eta 0.05, outflow, HLLC, van Leer; t = 0.12."""
    cfg = Config(nx=n, ny=n, nz=n, xl=-0.25, xr=0.25, yl=-0.25, yr=0.25, zl=-0.25, zr=0.25, gamma=5.0 / 3.0,
                 cfl=0.8, eta=0.5e-1, limiter=LIMITER_VANLEER, solver=SOLVER_HLLC, bc=(BC_OUTFLOW,) * 6)
    x, _, _ = cell_centres(cfg)  # the reference uses xcoord for all three axes
    s = -x[:, None, None] - x[None, :, None] - x[None, None, :]
    left = s > 0.0
    return cfg, conserved(cfg, np.where(left, 4.0, 1.0), 0.0, 0.0, 0.0, np.where(left, 1.0, 0.1795))


DIAG_SOD_TFIN = 0.12


def synthetic_cooling_table(n: int = 200, Tlo: float = 1e4, Thi: float = 1e8):
    """Piecewise power-law Lambda(T) on n log-spaced points over [1e4, 1e8] K:
    peak 10^-21.5 erg cm^3/s at 2e5 K, slope -0.7 up to 1e7 K, +0.5 above.
    Below the peak the slope anchors Lambda(1e4 K) at 10^-23.12, the first
    entry of the reference's Z1.0.dat table (slope ~ +1.245).  No cooling
    below 1e4 K (the table starts there).  Returns (T, log10 Lambda)."""
    T = np.logspace(np.log10(Tlo), np.log10(Thi), n)
    lt = np.log10(T)
    lpk, ltp = -21.5, np.log10(2e5)
    s_lo = (lpk - (-23.12)) / (ltp - np.log10(1e4))
    l7 = lpk - 0.7 * (7.0 - ltp)
    logL = np.where(lt < ltp, lpk + s_lo * (lt - ltp), np.where(lt <= 7.0, lpk - 0.7 * (lt - ltp), l7 + 0.5 * (lt - 7.0)))
    return T, logL


def wind_bubble(n: int = 256, cooling: int = COOL_SUBCYCLE, T_wind: float = 1.0e4, vw_kms: float = 2000.0,
                n_amb: float = 1.0, mdot_msun_yr: float = 1e-6, box_pc: float = 8.0, mass_msun: float = 10.0):
    """Radiative wind-blown bubble: n^3 in a (8 pc)^3 box centred on a
    spherical wind (radius 4 dx, Mdot 1e-6 Msun/yr, 2000 km/s, T_w 1e4 K) in an
    ambient medium n = 1 cm^-3, T = 1e4 K, mu = 1.3; gamma 5/3; synthetic
    cooling curve; a 10 Msun point mass at the origin; outflow; HLLC."""
    L = box_pc * PC
    T_cool, logL = synthetic_cooling_table()
    mu = 1.3
    cfg = Config(nx=n, ny=n, nz=n, xl=-L / 2, xr=L / 2, yl=-L / 2, yr=L / 2, zl=-L / 2, zr=L / 2, gamma=5.0 / 3.0,
                 cfl=0.4, eta=0.5e-2, mu0=mu, limiter=LIMITER_VANLEER, solver=SOLVER_HLLC, bc=(BC_OUTFLOW,) * 6,
                 cooling=cooling, cool_max_sub=16, cool_sub_frac=0.1, cool_T=T_cool, cool_logL=logL)
    cfg.winds = [Wind(xc=0.0, yc=0.0, zc=0.0, radius=4.0 * cfg.dx, mdot=mdot_msun_yr * MSUN / YEAR,
                      vinf=vw_kms * KMS, temp=T_wind, mu=mu)]
    cfg.masses = np.array([[0.0, 0.0, 0.0, mass_msun * MSUN]])
    rho = n_amb * mu * AMU
    # T = 1e4 K is the cooling table's first entry: cooling.f90:71 cools a
    # cell when temp >= cool_Tmin, so a medium at exactly 1e4 K is decided by
    # the last bit of its pressure.  1e-5 above the edge gives the
    # exact-arithmetic decision (cooled) robustly in every precision, FP32
    # included (its temperature carries ~1e-7 of rounding); the first step's
    # cooling then takes the medium ~4e-4 below the edge, where FP32 decides
    # too.
    p = n_amb * KB * 1.0e4 * (1.0 + 1e-5)
    return cfg, conserved(cfg, rho, 0.0, 0.0, 0.0, p)


def gravitating_cloud(n: int = 128, grav_bc: int = GBC_MULTIPOLE, box_pc: float = 4.0, radius_pc: float = 1.0,
                      n_cloud: float = 500.0, T_cloud: float = 50.0, contrast: float = 100.0, seed: int = 7,
                      mass_msun: float = 0.0):
    """A self-gravitating cloud (the reference's -DGRAV physics): a uniform
    sphere of radius 1 pc, n = 500 cm^-3 (mu 1.3), T = 50 K, in a 100 times
    thinner medium at the same pressure, in a (4 pc)^3 box of n^3 cells
    (n = 2^L, as MultiGrid needs); a 1 % seeded density perturbation breaks
    the symmetry; gamma 5/3, HLLC + van Leer, outflow, no cooling; optional
    point mass at the centre.  Free-fall time ~2 Myr."""
    L = box_pc * PC
    mu = 1.3
    cfg = Config(nx=n, ny=n, nz=n, xl=-L / 2, xr=L / 2, yl=-L / 2, yr=L / 2, zl=-L / 2, zr=L / 2, gamma=5.0 / 3.0,
                 cfl=0.4, eta=0.5e-2, mu0=mu, limiter=LIMITER_VANLEER, solver=SOLVER_HLLC, bc=(BC_OUTFLOW,) * 6,
                 self_gravity=1, grav_bc=grav_bc)
    if mass_msun > 0.0:
        cfg.masses = np.array([[0.0, 0.0, 0.0, mass_msun * MSUN]])
    x, y, z = cell_centres(cfg)
    X, Y, Z = np.meshgrid(x, y, z, indexing="ij")
    r = np.sqrt(X * X + Y * Y + Z * Z)
    rng = np.random.default_rng(seed)
    rho_c = n_cloud * mu * AMU
    inside = r < radius_pc * PC
    rho = np.where(inside, rho_c * (1.0 + 0.01 * rng.standard_normal(r.shape)), rho_c / contrast)
    p = n_cloud * KB * T_cloud  # pressure balance across the cloud's edge
    return cfg, conserved(cfg, rho, 0.0, 0.0, 0.0, p)


def random_state(cfg: Config, seed: int = 0, mach: float = 0.5, contrast: float = 0.3) -> np.ndarray:
    """Smooth-ish random valid state (rho, p > 0) for kernel-level parity."""
    rng = np.random.default_rng(seed)
    shp = cfg.shape[1:]
    rho = np.exp(contrast * rng.standard_normal(shp))
    p = np.exp(contrast * rng.standard_normal(shp))
    cs = np.sqrt(cfg.gamma * p / rho)
    v = [mach * cs * rng.standard_normal(shp) for _ in range(3)]
    return conserved(cfg, rho, v[0], v[1], v[2], p)


def periodic_box(n: int = 32):
    cfg = Config(nx=n, ny=n, nz=n, xl=0.0, xr=1.0, yl=0.0, yr=1.0, zl=0.0, zr=1.0, gamma=5.0 / 3.0, cfl=0.4,
                 bc=(BC_PERIODIC,) * 6)
    return cfg


def gaussian_field(n: int, seed: int, slope: float = -5.0 / 3.0) -> np.ndarray:
    """Periodic Gaussian random field on n^3 (zero mean, unit variance) whose
    shell-integrated power spectrum goes as k^slope (3-D amplitude
    k^((slope-2)/2)); k = 0 removed."""
    rng = np.random.default_rng(seed)
    k = np.fft.fftfreq(n) * n
    kz = np.fft.rfftfreq(n) * n
    kk = np.sqrt(k[:, None, None] ** 2 + k[None, :, None] ** 2 + kz[None, None, :] ** 2)
    kk[0, 0, 0] = 1.0
    amp = kk ** ((slope - 2.0) / 2.0)
    amp[0, 0, 0] = 0.0
    spec = amp * (rng.standard_normal(kk.shape) + 1j * rng.standard_normal(kk.shape))
    del kk, amp
    f = np.fft.irfftn(spec, s=(n, n, n), axes=(0, 1, 2))
    f -= f.mean()
    f /= f.std()
    return f


def clumpy(n: int = 384, seed: int = 0, cooling: int = COOL_SUBCYCLE, box_pc: float = 8.0, mach: float = 2.0,
           sigma_ln_n: float = 1.0, cool_max_sub: int = 16, cool_sub_frac: float = 0.1):
    """Clumpy radiative medium: n^3 periodic (8 pc)^3 box; a lognormal
    density, ln n Gaussian with standard deviation sigma_ln_n (k^-5/3
    spectrum), scaled to a mean of 1 cm^-3; log10 T uniform in [3, 8] (a
    k^-5/3 Gaussian field through its normal CDF); velocities k^-5/3 fields
    with rms Mach 2 relative to the 1e4 K sound speed; mu 1.3, gamma 5/3,
    HLLC, CFL 0.4; synthetic cooling curve."""
    from scipy.special import ndtr

    L = box_pc * PC
    T_cool, logL = synthetic_cooling_table()
    mu = 1.3
    cfg = Config(nx=n, ny=n, nz=n, xl=-L / 2, xr=L / 2, yl=-L / 2, yr=L / 2, zl=-L / 2, zr=L / 2, gamma=5.0 / 3.0,
                 cfl=0.4, eta=0.5e-2, mu0=mu, limiter=LIMITER_VANLEER, solver=SOLVER_HLLC, bc=(BC_PERIODIC,) * 6,
                 cooling=cooling, cool_max_sub=cool_max_sub, cool_sub_frac=cool_sub_frac, cool_T=T_cool,
                 cool_logL=logL)
    nd = np.exp(sigma_ln_n * gaussian_field(n, seed))
    nd /= nd.mean()
    lgT = 3.0 + 5.0 * ndtr(gaussian_field(n, seed + 1))
    cs4 = np.sqrt(cfg.gamma * KB * 1.0e4 / (mu * AMU))
    vel = [gaussian_field(n, seed + 2 + q) for q in range(3)]
    scale = mach * cs4 / np.sqrt(np.mean(vel[0] ** 2 + vel[1] ** 2 + vel[2] ** 2))
    rho_i = nd * mu * AMU
    p_i = nd * KB * 10.0 ** lgT
    del lgT, nd
    # interior fields; ghosts by periodic wrap (borders() refreshes them)
    wrap = lambda a: np.pad(a, 2, mode="wrap")
    return cfg, conserved(cfg, wrap(rho_i), *(wrap(scale * v) for v in vel), wrap(p_i))
