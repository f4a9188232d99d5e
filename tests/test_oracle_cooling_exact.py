"""The exact cooling integrator of the oracle (TLQO_COOL_EXACT), pinned
without the GPU.

The reference's apply_cooling (source/cooling.f90:47-119) takes one
exponential step; the sub-cycled integrator built on it (TLQO_COOL_SUBCYCLE)
converges, as its sub-steps shrink, to the solution of
d ln T/dt = -Lambda(T) n^2 / E_th at fixed density, and the exact integrator
is that limit in closed form (find_coef's log-linear interpolation,
cooling.f90:133-140, makes Lambda a piecewise power law).  Checked here:

* against an independent adaptive integration of the same equation
  (scipy's DOP853, relative tolerance 1e-12, Lambda from the oracle's own
  find_coef), over cells that stay in their table segment, cross many
  segments, reach the table's first temperature, or start above the table;
* that the sub-cycled integrator converges to it at first order;
* why it is the judge of the surrogate's energy error: on the clumpy medium
  the sub-cycled integrator with sub-steps of 2e-3 tau -- the previous
  "exact" integrator -- is itself 5e-6 of the total energy away from the
  limit after one step, 500 times the 1e-6 per 100 steps bar.
"""
import numpy as np
import pytest

from oracle.oracle import Oracle
from tests.helpers import oracle_params
from tlaloque_gb300 import problems, tlq

scipy_integrate = pytest.importorskip("scipy.integrate")


def _cool_oracle(cooling, frac=2e-3, max_sub=1):
    T, logL = problems.synthetic_cooling_table()
    cfg = tlq.Config(nx=4, ny=4, nz=4, cooling=cooling, cool_T=T, cool_logL=logL, cool_sub_frac=frac,
                     cool_max_sub=max_sub, mu0=1.3, gamma=5.0 / 3.0)
    return Oracle(oracle_params(cfg)), T


def _ode_T(o, T0_table, T, tau):
    """ln T(s) with d ln T/ds = -(Lambda(T)/T) / (Lambda(T_start)/T_start),
    s in [0, tau] (the cooling number's units), stopped at the table's first
    temperature."""
    c0 = o.cool_coef(T) / T

    def rhs(_s, y):
        Tc = np.exp(y[0])
        return [-(o.cool_coef(Tc) / Tc) / c0]

    def floor(_s, y):
        return y[0] - np.log(T0_table)
    floor.terminal = True
    floor.direction = -1
    sol = scipy_integrate.solve_ivp(rhs, (0.0, tau), [np.log(T)], method="DOP853", rtol=1e-12, atol=1e-14,
                                    events=floor, max_step=tau / 50)
    if sol.status == 1:
        return T0_table
    return float(np.exp(sol.y[0, -1]))


@pytest.mark.parametrize("T,tau", [
    (3.0e6, 1e-3),    # stays in its segment (slope -0.7)
    (5.0e4, 5e-3),    # rising branch (slope +1.245)
    (2.0e5, 0.3),     # the peak, crosses a few segments
    (1.0e7, 2.0),     # crosses many segments
    (4.0e4, 0.2),     # reaches 1e4 K within the step
    (2.0e8, 0.05),    # above the table (held at its last value)
    (1.0e4, 1e-2),    # at the first node
])
def test_exact_integrator_matches_adaptive_ode(T, tau):
    o, Tt = _cool_oracle(tlq.COOL_EXACT)
    got = o.cool_exact_T(T, tau)
    want = _ode_T(o, Tt[0], T, tau)
    assert got >= Tt[0]
    assert abs(got - want) <= 1e-9 * want, (got, want)


def test_subcycled_integrator_converges_to_exact_at_first_order():
    """Errors of the sub-cycled integrator against the closed form halve with
    the sub-step (first order), down to ~1e-6 relative."""
    T, tau = 3.0e5, 0.8
    o, _ = _cool_oracle(tlq.COOL_EXACT)
    exact = o.cool_exact_T(T, tau)
    errs = []
    for frac in (4e-3, 2e-3, 1e-3, 5e-4):
        cfg = _cell_cfg(tlq.COOL_SUBCYCLE, frac, 10 ** 6)
        errs.append(abs(_cool_one_cell(cfg, T, tau) - exact) / exact)
    ratios = [errs[q] / errs[q + 1] for q in range(3)]
    assert all(1.8 < r < 2.2 for r in ratios), (errs, ratios)
    assert errs[-1] < 5e-4


def _cell_cfg(cooling, frac, max_sub):
    Tt, logL = problems.synthetic_cooling_table()
    return tlq.Config(nx=2, ny=2, nz=2, xl=0.0, xr=1.0, yl=0.0, yr=1.0, zl=0.0, zr=1.0, cooling=cooling,
                      cool_T=Tt, cool_logL=logL, cool_sub_frac=frac, cool_max_sub=max_sub, mu0=1.3,
                      gamma=5.0 / 3.0)


def _cool_one_cell(cfg, T, tau):
    """T after one apply_cooling call on a uniform 2^3 mesh at density n = 1
    and temperature T, with dt chosen so that the cooling number is tau."""
    o = Oracle(oracle_params(cfg))
    rho = 1.3 * problems.AMU
    p = rho / (1.3 * problems.AMU) * problems.KB * T
    U = problems.conserved(cfg, rho, 0.0, 0.0, 0.0, p)
    W = o.calc_prims(U)
    ce = o.cool_coef(T) * 1.0 / (p / (cfg.gamma - 1.0))
    o.cooling(W, U, tau / ce)
    return float(W[4, 2, 2, 2] * 1.3 * problems.AMU / (W[0, 2, 2, 2] * problems.KB))


def test_exact_cell_step_single_and_closed_form():
    """One cell through apply_cooling: tau at most cool_sub_frac takes the
    reference's single exponential step (bit-identical to TLQO_COOL_REF),
    above it the closed form."""
    T = 2.5e6
    ref = _cool_one_cell(_cell_cfg(tlq.COOL_REF, 2e-3, 1), T, 1.5e-3)
    assert _cool_one_cell(_cell_cfg(tlq.COOL_EXACT, 2e-3, 1), T, 1.5e-3) == ref
    o, _ = _cool_oracle(tlq.COOL_EXACT)
    got = _cool_one_cell(_cell_cfg(tlq.COOL_EXACT, 2e-3, 1), T, 0.4)
    assert abs(got - o.cool_exact_T(T, 0.4)) <= 1e-12 * got


def test_subcycled_judge_error_carries_the_clumpy_energy_drift():
    """On the clumpy medium (48^3), one cooling call with the CFL step: the
    sub-cycled integrator at sub-steps of 2e-3 tau differs from the exact
    integrator by ~5e-8 of the total energy -- over 100 steps several times
    the 1e-6 bar, whatever a surrogate does -- and halves with the
    sub-step."""
    cfg, U0 = problems.clumpy(48)
    out = {}
    for cooling, frac, msub in ((tlq.COOL_EXACT, 2e-3, 1), (tlq.COOL_SUBCYCLE, 2e-3, 20000),
                                (tlq.COOL_SUBCYCLE, 1e-3, 40000)):
        c = tlq.Config(**{**cfg.__dict__, "cooling": cooling, "cool_sub_frac": frac, "cool_max_sub": msub})
        o = Oracle(oracle_params(c, nthreads=4))
        U = U0.copy(order="F")
        o.borders(U, 1)
        W = o.calc_prims(U)
        dt = o.time_step(W)
        o.cooling(W, U, dt)
        out[(cooling, frac)] = U[4, 2:-2, 2:-2, 2:-2].sum()
    E = out[(tlq.COOL_EXACT, 2e-3)]
    d2 = (out[(tlq.COOL_SUBCYCLE, 2e-3)] - E) / E
    d1 = (out[(tlq.COOL_SUBCYCLE, 1e-3)] - E) / E
    assert 100 * d2 > 2e-6    # under-cools: the sub-steps take the coefficient at their start
    assert 1.7 < d2 / d1 < 2.3
