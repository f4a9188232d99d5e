"""Pin the CPU oracle (and the analysis tools) against the reference's golden
data and analytic solutions.  CPU only."""
import numpy as np
import pytest

from oracle.oracle import Run
from tests.helpers import oracle_params
from tlaloque_gb300 import analysis, problems

pytestmark = pytest.mark.timeout(600)


def test_exact_riemann_reproduces_reference_sod_file(golden):
    """The exact Riemann solver against solutions/sod_e1rpex.out (the exact
    solution the reference's Sod analysis plots, tests_analisis.jl:77-85):
    rho 4, p 1 | rho 1, p 0.1795, gamma 5/3, t = 0.12, x in [-0.25, 0.25]."""
    ref = golden["sod_e1rpex"]
    x = ref[:, 0] - 0.25
    rho, u, p = analysis.riemann_sample(4.0, 0.0, 1.0, 1.0, 0.0, 0.1795, 5.0 / 3.0, x / 0.12)
    e = p / ((5.0 / 3.0 - 1.0) * rho)
    # the file has 6 decimals; away from the (sampled) discontinuities the
    # two agree to its precision
    for col, mine in ((1, rho), (2, u), (3, p), (4, e)):
        err = np.abs(mine - ref[:, col])
        assert np.median(err) < 2e-6
        assert np.mean(err < 1e-5) > 0.99


def _diag_sod_metrics(n):
    cfg, U0 = problems.diagonal_sod(n)
    run = Run(oracle_params(cfg), U0)
    run.run(10 ** 6, problems.DIAG_SOD_TFIN)
    r, rho, vel, p, e = analysis.diagonal_profiles(cfg, run.UPrim)
    return run, r, rho, vel, p, e


def test_oracle_diagonal_sod_against_reference_solution(golden):
    """The reference's own Sod test (tests_utilities.jl:214-224) on the oracle
    at reduced resolution, scored with the reference's metrics
    (utils_analisis.jl:23-72) against its exact-solution file."""
    ref = golden["sod_e1rpex"]
    xex = ref[:, 0] - 0.25
    run, r, rho, vel, p, e = _diag_sod_metrics(64)
    # the loop has no last-step clamp (mainHD.f90:61): t overshoots tfin
    assert run.t >= problems.DIAG_SOD_TFIN and run.t < problems.DIAG_SOD_TFIN + 0.01
    _, mape_d, _, L1_d, L2_d, _ = analysis.all_error_metrics(xex, ref[:, 1], r, rho)
    _, _, _, L1_p, _, _ = analysis.all_error_metrics(xex, ref[:, 3], r, p)
    _, _, _, L1_v, _, _ = analysis.all_error_metrics(xex, ref[:, 2], r, vel)
    _, _, _, L1_e, _, _ = analysis.all_error_metrics(xex, ref[:, 4], r, e)
    # 64^3 values: rho 0.031, p 0.034, |v| 0.156, e 0.031 (they fall with n)
    assert L1_d < 0.04 and L1_p < 0.045 and L1_v < 0.2 and L1_e < 0.04
    assert mape_d < 0.05


def test_oracle_sod_tube_against_exact_solution():
    """Classic Sod (256x4x4, HLL, gamma 1.4) to t = 0.2 against the exact
    Riemann solution."""
    cfg, U0 = problems.sod_tube()
    run = Run(oracle_params(cfg), U0)
    run.run(10 ** 6, problems.SOD_TFIN)
    W = run.UPrim
    x = cfg.xl + cfg.dx * (np.arange(cfg.nx) + 0.5)
    rho_num = W[0, 2:-2, 4, 4]
    rho_ex, u_ex, p_ex = analysis.sod_exact(x, run.t)
    # HLL at 256 cells: L1(rho) = 0.020 (HLLC: 0.013)
    assert analysis.norm_L1(rho_ex, rho_num) < 0.025
    assert analysis.norm_L1(p_ex, W[4, 2:-2, 4, 4]) < 0.025
    # Transverse cells differ only by the viscosity term next to the y/z
    # faces: `step` fills U's ghosts from the pre-viscosity UP
    # (HydroCore.f90:195-206), so a face-adjacent cell's 7-point stencil sees
    # UP there while interior neighbours hold the viscous U.
    spread = np.max(np.abs(W[0, 2:-2, 2:-2, 2:-2] - rho_num[:, None, None]))
    assert 0.0 < spread < 1e-4


def test_oracle_sedov_shock_radius_and_profile(golden):
    """Sedov-Taylor blast (gamma 5/3) at reduced resolution: shock radius and
    density profile against the similarity solution
    (solutions/sedov_solution_53.txt)."""
    cfg, U0 = problems.sedov(48)
    run = Run(oracle_params(cfg), U0)
    run.run(10 ** 6, problems.SEDOV_TFIN)
    t = run.t
    Rs = problems.sedov_shock_radius(t, xi0=float(golden["sedov53_xi0"]))
    rc, prof = analysis.radial_profile(cfg, run.UPrim[0, 2:-2, 2:-2, 2:-2], nbins=24, rmax=0.48)
    ok = np.isfinite(prof)
    r_peak = rc[ok][np.argmax(prof[ok])]
    assert abs(r_peak - Rs) < 2.5 * cfg.dx
    exact = analysis.sedov_density(rc, t, golden["sedov53"])
    inner = ok & (rc < 1.2 * Rs)
    # L1(rho) 0.41 / 0.34 / 0.30 at 32^3 / 48^3 / 64^3 (the shell is under-resolved)
    assert analysis.norm_L1(exact[inner], prof[inner]) < 0.36
    # total energy: E0 plus the background's p0/(gamma-1) volume, conserved
    # while the blast stays inside the box
    E = run.U[4, 2:-2, 2:-2, 2:-2].sum() * cfg.dx ** 3
    assert abs(E - (1.0 + 1e-5 / (2.0 / 3.0))) < 1e-6


def test_cooling_table_z1_lookup(golden):
    """find_coef (cooling.f90:121-144) on the reference's Z1.0.dat table:
    exact at the nodes, log-linear between, held at the last node above."""
    from oracle.oracle import COOL_REF, Oracle, Params
    T = golden["z1_T"]
    logL = -golden["z1_b"]
    o = Oracle(Params(nx=4, ny=4, nz=4, cooling=COOL_REF, cool_T=T, cool_logL=logL))
    for q in (0, 10, 250, 499):
        assert o.cool_coef(T[q]) == pytest.approx(10.0 ** logL[q], rel=1e-12)
    mid = np.sqrt(T[100] * T[101])
    assert o.cool_coef(mid) == pytest.approx(10.0 ** (0.5 * (logL[100] + logL[101])), rel=1e-12)
    assert o.cool_coef(2 * T[-1]) == pytest.approx(10.0 ** logL[-1], rel=1e-12)
