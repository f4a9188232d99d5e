"""The synthetic workloads (tlaloque_gb300/problems.py) have the shapes, sizes
and value distributions their definitions state: the inputs of the
benchmarks, checked on the CPU at small sizes."""
import numpy as np
import pytest

from tlaloque_gb300 import problems as P
from tlaloque_gb300 import tlq


def prims(cfg, U):
    """(rho, vx, vy, vz, p) of U in the reference layout."""
    rho = U[0]
    v = [U[e] / rho for e in (1, 2, 3)]
    ek = 0.5 * rho * (v[0] ** 2 + v[1] ** 2 + v[2] ** 2)
    return rho, v[0], v[1], v[2], (cfg.gamma - 1.0) * (U[4] - ek)


def interior(a):
    return a[..., 2:-2, 2:-2, 2:-2]


def test_sod_tube_states():
    cfg, U = P.sod_tube()
    assert (cfg.nx, cfg.ny, cfg.nz) == (256, 4, 4) and cfg.gamma == 1.4 and cfg.solver == tlq.SOLVER_HLL
    assert U.shape == cfg.shape
    assert np.isclose(cfg.dy, cfg.dx) and np.isclose(cfg.dz, cfg.dx)
    rho, vx, _, _, p = prims(cfg, U)
    x, _, _ = P.cell_centres(cfg)
    left = x < 0.5
    assert np.all(rho[left] == 1.0) and np.all(rho[~left] == 0.125)
    assert np.allclose(p[left], 1.0) and np.allclose(p[~left], 0.1)
    assert np.all(vx == 0.0)


def test_sedov_deposits_exactly_E0():
    """E0 = 1 as thermal energy, uniform over the interior cells whose centre
    lies within 3 dx of the origin: their energy sums to E0 to round-off."""
    n = 32
    cfg, U = P.sedov(n)
    x, y, z = P.cell_centres(cfg)
    r = np.sqrt(x[:, None, None] ** 2 + y[None, :, None] ** 2 + z[None, None, :] ** 2)
    inside = interior(r) < 3.0 * cfg.dx
    dV = cfg.dx * cfg.dy * cfg.dz
    E = interior(U[4])
    assert abs(np.sum(E[inside]) * dV - 1.0) < 1e-12
    assert np.allclose(interior(U[0]), 1.0)
    p0 = 1e-5 / (cfg.gamma - 1.0)
    assert np.allclose(E[~inside], p0)


def test_diagonal_sod_states():
    cfg, U = P.diagonal_sod(16)
    rho, _, _, _, p = prims(cfg, U)
    x, _, _ = P.cell_centres(cfg)
    s = -x[:, None, None] - x[None, :, None] - x[None, None, :]
    assert np.all(rho[s > 0] == 4.0) and np.all(rho[s <= 0] == 1.0)
    assert np.allclose(p[s > 0], 1.0) and np.allclose(p[s <= 0], 0.1795)


def test_synthetic_cooling_table_anchors():
    T, logL = P.synthetic_cooling_table()
    assert len(T) == 200 and np.isclose(T[0], 1e4) and np.isclose(T[-1], 1e8)
    assert np.all(np.diff(T) > 0)
    assert np.isclose(logL[0], -23.12)  # the first entry of the reference's Z1.0.dat
    lt = np.log10(T)
    # continuous at the peak (2e5 K, 10^-21.5) and at 1e7 K
    f = lambda t: np.interp(np.log10(t), lt, logL)
    assert abs(f(2e5) - (-21.5)) < 2e-2
    assert logL.max() <= -21.5 + 1e-12
    below, above = f(1e7 * 0.999), f(1e7 * 1.001)
    assert abs(below - above) < 2e-3


def test_wind_bubble_definition():
    n = 32
    cfg, U = P.wind_bubble(n)
    L = 8.0 * P.PC
    assert np.isclose(cfg.xr - cfg.xl, L) and np.isclose(cfg.dx, L / n)
    assert cfg.cooling == tlq.COOL_SUBCYCLE and cfg.solver == tlq.SOLVER_HLLC and cfg.gamma == 5.0 / 3.0
    (w,) = cfg.winds
    assert np.isclose(w.radius, 4.0 * cfg.dx) and np.isclose(w.vinf, 2000.0 * P.KMS)
    assert np.isclose(w.mdot, 1e-6 * P.MSUN / P.YEAR) and w.temp == 1.0e4
    assert np.isclose(cfg.masses[0, 3], 10.0 * P.MSUN) and np.all(cfg.masses[0, :3] == 0.0)
    rho, vx, vy, vz, p = prims(cfg, U)
    assert np.allclose(rho, 1.3 * P.AMU)
    T = p * 1.3 * P.AMU / (rho * P.KB)
    assert np.allclose(T, 1.0e4, rtol=2e-5) and np.all(T > 1.0e4)  # just above the table's first entry
    assert np.all(vx == 0.0) and np.all(vy == 0.0) and np.all(vz == 0.0)


def test_gaussian_field_moments_and_spectrum():
    n = 64
    f = P.gaussian_field(n, seed=3)
    assert abs(f.mean()) < 1e-12 and abs(f.std() - 1.0) < 1e-12
    # shell-integrated power ~ k^(-5/3): fitted slope over 2 <= k <= n/4
    F = np.abs(np.fft.fftn(f)) ** 2
    k = np.fft.fftfreq(n) * n
    kk = np.sqrt(k[:, None, None] ** 2 + k[None, :, None] ** 2 + k[None, None, :] ** 2)
    shells = np.arange(2, n // 4)
    power = np.array([F[(kk >= s - 0.5) & (kk < s + 0.5)].sum() for s in shells])
    slope = np.polyfit(np.log(shells), np.log(power), 1)[0]
    assert abs(slope - (-5.0 / 3.0)) < 0.25


def test_clumpy_medium_distributions():
    pytest.importorskip("scipy")
    n = 32
    cfg, U = P.clumpy(n, seed=1)
    assert all(b == tlq.BC_PERIODIC for b in cfg.bc)
    rho, vx, vy, vz, p = prims(cfg, U)
    nd = interior(rho) / (1.3 * P.AMU)
    # lognormal density: sigma(ln n) = 1, mean 1 cm^-3
    assert abs(np.log(nd).std() - 1.0) < 1e-9 and abs(nd.mean() - 1.0) < 1e-9
    T = interior(p) * 1.3 * P.AMU / (interior(rho) * P.KB)
    assert T.min() >= 1e3 * (1 - 1e-9) and T.max() <= 1e8 * (1 + 1e-9)
    cs4 = np.sqrt(cfg.gamma * P.KB * 1.0e4 / (1.3 * P.AMU))
    v2 = interior(vx) ** 2 + interior(vy) ** 2 + interior(vz) ** 2
    assert abs(np.sqrt(v2.mean()) / cs4 - 2.0) < 1e-9  # rms Mach 2 against the 1e4 K sound speed
    # ghosts: the periodic wrap of the interior
    assert np.array_equal(U[:, :2, 2:-2, 2:-2], U[:, -4:-2, 2:-2, 2:-2])
    assert np.array_equal(U[:, 2:-2, 2:-2, -2:], U[:, 2:-2, 2:-2, 2:4])


@pytest.mark.parametrize("grav_bc", [tlq.GBC_ZERO, tlq.GBC_MULTIPOLE])
def test_gravitating_cloud_definition(grav_bc):
    n = 32
    cfg, U = P.gravitating_cloud(n, grav_bc=grav_bc)
    assert cfg.self_gravity == 1 and cfg.grav_bc == grav_bc and cfg.nx == cfg.ny == cfg.nz == n
    assert n & (n - 1) == 0  # a cube of 2^L cells, as MultiGrid needs
    x, y, z = P.cell_centres(cfg)
    r = np.sqrt(x[:, None, None] ** 2 + y[None, :, None] ** 2 + z[None, None, :] ** 2)
    rho, _, _, _, p = prims(cfg, U)
    rho_c = 500.0 * 1.3 * P.AMU
    inside = r < 1.0 * P.PC
    assert np.all(np.abs(rho[inside] / rho_c - 1.0) < 0.1)  # 1 % seeded perturbation
    assert abs(rho[inside].mean() / rho_c - 1.0) < 2e-3
    assert np.allclose(rho[~inside], rho_c / 100.0)
    assert np.allclose(p, 500.0 * P.KB * 50.0)  # pressure balance across the edge
