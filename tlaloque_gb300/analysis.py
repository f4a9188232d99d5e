"""Analysis tools of the reference's test harness, restated in Python.

* error metrics MAPE / RMSPE / L1 / L2 / Linf with piecewise-linear
  interpolation of the exact profile (utils_analisis.jl:1-94);
* diagonal profiles of a cube (tests_analisis.jl:64-71);
* an exact Riemann solver for the Euler equations (ideal gas), written from
  the standard pressure-function / Newton formulation (Toro, "Riemann Solvers
  and Numerical Methods for Fluid Dynamics", ch. 4);
* radial binning for the Sedov-Taylor comparison.
"""
from __future__ import annotations

import math

import numpy as np


# ---------------------------------------------------------------------------
# utils_analisis.jl
# ---------------------------------------------------------------------------
def radius_sedov(t: float, E0: float, rho0: float) -> float:
    """utils_analisis.jl:1-3."""
    return 1.15 * (E0 * t ** 2 / rho0) ** (1 / 5)


def all_error_metrics(xex, yex, xnum, ynum):
    """_all_error_metrics (utils_analisis.jl:23-72): interpolate the exact
    profile (xex ascending) at the numerical abscissae inside its range.
    Returns (rel_errors, MAPE, RMSPE, L1, L2, Linf) or Nones when a point
    falls outside the exact table."""
    xex = np.asarray(xex, float)
    yex = np.asarray(yex, float)
    xnum = np.asarray(xnum, float)
    ynum = np.asarray(ynum, float)
    idx = int(np.argmax(xnum >= xex[0])) if xex[0] > xnum[0] else 0
    fdx = int(np.nonzero(xnum <= xex[-1])[0][-1]) if xex[-1] < xnum[-1] else len(xnum) - 1
    scale = np.max(np.abs(yex))
    errs = []
    mape = rmspe = L1n = L1d = L2n = L2d = 0.0
    k = 1
    for i in range(idx, fdx + 1):
        # _neighbor_search: first exact node beyond xnum[i], scanning from k
        kk = None
        for q in range(k, len(xex)):
            if xex[q] > xnum[i]:
                kk = q
                break
        if kk is None:
            return None, None, None, None, None, None
        j, k = kk - 1, kk
        m = (yex[k] - yex[j]) / (xex[k] - xex[j])
        b = (xex[k] * yex[j] - yex[k] * xex[j]) / (xex[k] - xex[j])
        yi = m * xnum[i] + b
        ea = abs(yi - ynum[i])
        er = ea / abs(yi) if abs(yi) > 1e-12 else ea / scale
        errs.append(er)
        mape += er
        rmspe += er * er
        L1n += ea
        L1d += abs(yi)
        L2n += ea * ea
        L2d += yi * yi
    n = len(errs)
    return np.array(errs), mape / n, math.sqrt(rmspe / n), L1n / L1d, math.sqrt(L2n / L2d), max(errs)


def norm_L1(yex, ynum) -> float:
    yex, ynum = np.asarray(yex), np.asarray(ynum)
    return float(np.sum(np.abs(yex - ynum)) / np.sum(np.abs(yex)))


def norm_L2(yex, ynum) -> float:
    yex, ynum = np.asarray(yex), np.asarray(ynum)
    return float(np.sqrt(np.sum((yex - ynum) ** 2) / np.sum(yex ** 2)))


def norm_Linf(yex, ynum) -> float:
    yex, ynum = np.asarray(yex), np.asarray(ynum)
    return float(np.max(np.abs(yex - ynum)) / np.max(np.abs(yex)))


# ---------------------------------------------------------------------------
# Diagonal profiles (tests_analisis.jl:64-71): r = sign(x) sqrt(3) |x| along
# the main diagonal (i, i, i) of an n^3 cube (interior cells).
# ---------------------------------------------------------------------------
def diagonal_profiles(cfg, W):
    n = cfg.nx
    idx = np.arange(2, n + 2)
    x = cfg.xl + cfg.dx * np.arange(1, n + 1) - cfg.dx / 2.0
    r = np.sign(x) * np.sqrt(3.0 * x * x)
    rho = W[0, idx, idx, idx]
    p = W[4, idx, idx, idx]
    vel = np.sqrt(W[1, idx, idx, idx] ** 2 + W[2, idx, idx, idx] ** 2 + W[3, idx, idx, idx] ** 2)
    e = p / ((cfg.gamma - 1.0) * rho)
    return r, rho, vel, p, e


# ---------------------------------------------------------------------------
# Exact Riemann solver (ideal gas).
# ---------------------------------------------------------------------------
def _fK(p, rhoK, pK, cK, g):
    """Pressure function f_K and derivative (shock for p > pK, rarefaction otherwise)."""
    if p > pK:
        A = 2.0 / ((g + 1.0) * rhoK)
        B = (g - 1.0) / (g + 1.0) * pK
        q = math.sqrt(A / (p + B))
        return (p - pK) * q, q * (1.0 - 0.5 * (p - pK) / (B + p))
    e = (g - 1.0) / (2.0 * g)
    f = 2.0 * cK / (g - 1.0) * ((p / pK) ** e - 1.0)
    return f, 1.0 / (rhoK * cK) * (p / pK) ** (-(g + 1.0) / (2.0 * g))


def riemann_star(rL, uL, pL, rR, uR, pR, g):
    """Star-region pressure and velocity (Newton iteration on f_L + f_R + du = 0)."""
    cL, cR = math.sqrt(g * pL / rL), math.sqrt(g * pR / rR)
    du = uR - uL
    if 2.0 * (cL + cR) / (g - 1.0) <= du:
        raise ValueError("vacuum is generated")
    # two-rarefaction guess
    e = (g - 1.0) / (2.0 * g)
    p = ((cL + cR - 0.5 * (g - 1.0) * du) / (cL / pL ** e + cR / pR ** e)) ** (1.0 / e)
    p = max(p, 1e-12 * min(pL, pR))
    for _ in range(100):
        fL, dL = _fK(p, rL, pL, cL, g)
        fR, dR = _fK(p, rR, pR, cR, g)
        pn = p - (fL + fR + du) / (dL + dR)
        pn = max(pn, 1e-14 * min(pL, pR))
        if abs(pn - p) <= 1e-14 * 0.5 * (pn + p):
            p = pn
            break
        p = pn
    fL, _ = _fK(p, rL, pL, cL, g)
    fR, _ = _fK(p, rR, pR, cR, g)
    u = 0.5 * (uL + uR) + 0.5 * (fR - fL)
    return p, u


def riemann_sample(rL, uL, pL, rR, uR, pR, g, s):
    """Exact solution (rho, u, p) at similarity coordinates s = (x - x0)/t."""
    s = np.atleast_1d(np.asarray(s, float))
    ps, us = riemann_star(rL, uL, pL, rR, uR, pR, g)
    cL, cR = math.sqrt(g * pL / rL), math.sqrt(g * pR / rR)
    gm, gp = (g - 1.0) / (g + 1.0), 2.0 / (g + 1.0)
    out = np.zeros((3, s.size))
    for q, S in enumerate(s):
        if S <= us:  # left of the contact
            if ps > pL:  # left shock
                SL = uL - cL * math.sqrt((g + 1.0) / (2.0 * g) * ps / pL + (g - 1.0) / (2.0 * g))
                if S <= SL:
                    out[:, q] = (rL, uL, pL)
                else:
                    rs = rL * ((ps / pL + gm) / (gm * ps / pL + 1.0))
                    out[:, q] = (rs, us, ps)
            else:  # left rarefaction
                SHL = uL - cL
                csL = cL * (ps / pL) ** ((g - 1.0) / (2.0 * g))
                STL = us - csL
                if S <= SHL:
                    out[:, q] = (rL, uL, pL)
                elif S >= STL:
                    out[:, q] = (rL * (ps / pL) ** (1.0 / g), us, ps)
                else:
                    c = gp * (cL + 0.5 * (g - 1.0) * (uL - S))
                    u = gp * (cL + 0.5 * (g - 1.0) * uL + S)
                    rho = rL * (c / cL) ** (2.0 / (g - 1.0))
                    out[:, q] = (rho, u, pL * (c / cL) ** (2.0 * g / (g - 1.0)))
        else:  # right of the contact
            if ps > pR:  # right shock
                SR = uR + cR * math.sqrt((g + 1.0) / (2.0 * g) * ps / pR + (g - 1.0) / (2.0 * g))
                if S >= SR:
                    out[:, q] = (rR, uR, pR)
                else:
                    rs = rR * ((ps / pR + gm) / (gm * ps / pR + 1.0))
                    out[:, q] = (rs, us, ps)
            else:  # right rarefaction
                SHR = uR + cR
                csR = cR * (ps / pR) ** ((g - 1.0) / (2.0 * g))
                STR = us + csR
                if S >= SHR:
                    out[:, q] = (rR, uR, pR)
                elif S <= STR:
                    out[:, q] = (rR * (ps / pR) ** (1.0 / g), us, ps)
                else:
                    c = gp * (cR - 0.5 * (g - 1.0) * (uR - S))
                    u = gp * (-cR + 0.5 * (g - 1.0) * uR + S)
                    rho = rR * (c / cR) ** (2.0 / (g - 1.0))
                    out[:, q] = (rho, u, pR * (c / cR) ** (2.0 * g / (g - 1.0)))
    return out


def sod_exact(x, t, x0=0.5, left=(1.0, 0.0, 1.0), right=(0.125, 0.0, 0.1), g=1.4):
    """(rho, u, p) of a shock tube at positions x and time t."""
    x = np.asarray(x, float)
    return riemann_sample(*left, *right, g, (x - x0) / t)


# ---------------------------------------------------------------------------
# Sedov-Taylor: radial profile of a cube and the similarity solution.
# ---------------------------------------------------------------------------
def radial_profile(cfg, field_interior: np.ndarray, centre=(0.0, 0.0, 0.0), nbins: int = 64, rmax: float | None = None):
    """Mean of an interior field in radial shells around `centre`."""
    x = cfg.xl + cfg.dx * (np.arange(cfg.nx) + 0.5)
    y = cfg.yl + cfg.dy * (np.arange(cfg.ny) + 0.5)
    z = cfg.zl + cfg.dz * (np.arange(cfg.nz) + 0.5)
    r = np.sqrt((x[:, None, None] - centre[0]) ** 2 + (y[None, :, None] - centre[1]) ** 2 +
                (z[None, None, :] - centre[2]) ** 2)
    rmax = rmax if rmax is not None else float(min(cfg.xr - centre[0], centre[0] - cfg.xl))
    edges = np.linspace(0.0, rmax, nbins + 1)
    which = np.digitize(r.ravel(), edges) - 1
    ok = (which >= 0) & (which < nbins)
    cnt = np.bincount(which[ok], minlength=nbins)
    s = np.bincount(which[ok], weights=field_interior.ravel()[ok], minlength=nbins)
    rc = 0.5 * (edges[1:] + edges[:-1])
    with np.errstate(invalid="ignore", divide="ignore"):
        return rc, s / cnt


def sedov_density(r, t, table, E0=1.0, rho0=1.0, gamma=5.0 / 3.0):
    """Analytic rho(r) from a similarity table with columns (xi, rho/rho_1)
    (solutions/sedov_solution_53.txt columns 1-2); rho_1 = rho0 (g+1)/(g-1)."""
    xi_tab = np.asarray(table[:, 0])
    a_tab = np.asarray(table[:, 1])
    order = np.argsort(xi_tab)
    xi_tab, a_tab = xi_tab[order], a_tab[order]
    L = (E0 * t * t / rho0) ** 0.2
    xi = np.asarray(r) / L
    rho1 = rho0 * (gamma + 1.0) / (gamma - 1.0)
    return np.where(xi <= xi_tab[-1], rho1 * np.interp(xi, xi_tab, a_tab), rho0)
