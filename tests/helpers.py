"""Shared test helpers: mirror a package Config into oracle Params, compare
arrays on the cells the scheme defines."""
import numpy as np

from oracle.oracle import Params, Wind as OWind


def oracle_params(cfg, nthreads: int = 0) -> Params:
    p = Params(nx=cfg.nx, ny=cfg.ny, nz=cfg.nz, xl=cfg.xl, xr=cfg.xr, yl=cfg.yl, yr=cfg.yr, zl=cfg.zl, zr=cfg.zr,
               gamma=cfg.gamma, cfl=cfg.cfl, eta=cfg.eta, mu0=cfg.mu0, cooling_limit=cfg.cooling_limit,
               limiter=cfg.limiter, solver=cfg.solver, bc=tuple(cfg.bc), cooling=cfg.cooling,
               cool_T=cfg.cool_T, cool_logL=cfg.cool_logL, cool_max_sub=cfg.cool_max_sub,
               cool_sub_frac=cfg.cool_sub_frac, nthreads=nthreads)
    p.winds = [OWind(**{k: getattr(w, k) for k in ("xc", "yc", "zc", "vx", "vy", "vz", "radius", "mdot", "vinf",
                                                    "temp", "mu")}) for w in cfg.winds]
    p.masses = None if cfg.masses is None else np.asarray(cfg.masses, float)
    p.plane_winds = list(getattr(cfg, "plane_winds", []))
    p.self_gravity = int(getattr(cfg, "self_gravity", 0))
    p.grav_bc = int(getattr(cfg, "grav_bc", 0))
    return p


def interior(a):
    return a[:, 2:-2, 2:-2, 2:-2]


def face_ghost_mask(cfg):
    """Cells the step defines: the interior and the first ghost layer of each
    face (transverse indices interior)."""
    m = np.zeros(cfg.shape[1:], bool)
    m[2:-2, 2:-2, 2:-2] = True
    m[1, 2:-2, 2:-2] = m[-2, 2:-2, 2:-2] = True
    m[2:-2, 1, 2:-2] = m[2:-2, -2, 2:-2] = True
    m[2:-2, 2:-2, 1] = m[2:-2, 2:-2, -2] = True
    return m


def rel_l1(a, b):
    """Relative L1 difference per conserved variable over the given cells."""
    return np.array([np.sum(np.abs(a[e] - b[e])) / max(np.sum(np.abs(b[e])), 1e-300) for e in range(a.shape[0])])
