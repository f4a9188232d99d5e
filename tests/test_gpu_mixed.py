"""Mixed-precision step (FP32 reconstruction, Riemann fluxes, sources and
cooling; FP64 accumulation, high-Mach pressure recovery and dt) against the
plain FP64 step.  The plain step is bit-identical to the oracle (its own
tests), so it stands in for the oracle on runs too long for the CPU.

Bars (the mixed form's targets): relative L1 density error <= 1 % and relative
total-energy drift <= 1e-6 per 100 steps against FP64; short runs are held
much tighter (they are FP32 round-off only)."""
import numpy as np
import pytest

from oracle.oracle import Run
from tests.helpers import interior, oracle_params
from tests.test_gpu_step import smooth_state
from tlaloque_gb300 import analysis, problems, tlq

pytestmark = pytest.mark.gpu


def run_gpu(cfg, U0, nsteps=None, tfin=None, precision=tlq.PREC_FP64):
    cfg = tlq.Config(**{**cfg.__dict__, "precision": precision})
    U1 = U0.copy(order="F")
    with tlq.Context(cfg) as ctx:
        ctx.borders(U1, 1)
        ctx.upload(U1)
        if tfin is not None:
            ctx.run_until(tfin)
        else:
            ctx.advance(nsteps)
        t, it, dt, rc = ctx.time()
        U, W = ctx.state()
        sums = ctx.conserved_sums()
    return U, W, (t, it, dt, rc), sums


def rel_l1(a, b):
    return float(np.sum(np.abs(a - b)) / np.sum(np.abs(b)))


@pytest.mark.parametrize("limiter", [tlq.LIMITER_VANLEER, tlq.LIMITER_MINMOD, tlq.LIMITER_SUPERBEE])
def test_mixed_short_run_against_oracle(gpu_lib, limiter):
    cfg = tlq.Config(nx=33, ny=20, nz=24, xl=0.0, xr=1.0, yl=0.0, yr=0.6, zl=0.0, zr=0.7, limiter=limiter,
                     bc=(tlq.BC_REFLECTIVE, tlq.BC_OUTFLOW, tlq.BC_PERIODIC, tlq.BC_PERIODIC, tlq.BC_OUTFLOW,
                         tlq.BC_REFLECTIVE))
    U0 = smooth_state(cfg, seed=limiter, mach=1.1)
    run = Run(oracle_params(cfg), U0)
    run.run(10)
    U, W, (t, it, dt, rc), _ = run_gpu(cfg, U0, 10, precision=tlq.PREC_MIXED)
    assert rc == tlq.OK and it == run.it
    err = [rel_l1(interior(U)[e], interior(run.U)[e]) for e in range(5)]
    # FP32 round-off on a Mach ~1 random field, 10 steps (the bar is 1 %;
    # superbee, the most compressive limiter, amplifies it most)
    assert max(err) < 1e-3, err
    assert abs(t - run.t) < 1e-5 * run.t


def test_mixed_wind_bubble_100_steps_bars(gpu_lib):
    """Wind bubble (wind, point mass, sub-cycled cooling) at 64^3, 100 steps:
    L1 density error <= 1 % and total-energy drift <= 1e-6 against FP64."""
    cfg, U0 = problems.wind_bubble(64)
    U64, W64, (t64, it64, _, rc64), s64 = run_gpu(cfg, U0, 100, precision=tlq.PREC_FP64)
    Um, Wm, (tm, itm, _, rcm), sm = run_gpu(cfg, U0, 100, precision=tlq.PREC_MIXED)
    assert rc64 == tlq.OK and rcm == tlq.OK and it64 == itm == 100
    err = rel_l1(interior(Wm)[0], interior(W64)[0])
    assert err <= 1e-2, err
    # total energy: compare the two runs at the same simulated time
    drift = abs(sm[4] - s64[4]) / abs(s64[4])
    assert drift <= 1e-6 * max(1.0, 100 / 100), (drift, sm[4], s64[4])
    assert abs(tm - t64) <= 1e-4 * t64


def test_mixed_sod_tube_against_exact(gpu_lib):
    cfg, U0 = problems.sod_tube()
    U, W, (t, it, dt, rc), _ = run_gpu(cfg, U0, tfin=problems.SOD_TFIN, precision=tlq.PREC_MIXED)
    x = cfg.xl + cfg.dx * (np.arange(cfg.nx) + 0.5)
    rho_ex, u_ex, p_ex = analysis.sod_exact(x, t)
    assert analysis.norm_L1(rho_ex, W[0, 2:-2, 4, 4]) < 0.025


def test_mixed_sedov_shock_radius(gpu_lib, golden):
    cfg, U0 = problems.sedov(64)
    U, W, (t, it, dt, rc), _ = run_gpu(cfg, U0, tfin=problems.SEDOV_TFIN, precision=tlq.PREC_MIXED)
    U64, W64, _, _ = run_gpu(cfg, U0, tfin=problems.SEDOV_TFIN, precision=tlq.PREC_FP64)
    Rs = problems.sedov_shock_radius(t, xi0=float(golden["sedov53_xi0"]))
    rc_, prof = analysis.radial_profile(cfg, W[0, 2:-2, 2:-2, 2:-2], nbins=32, rmax=0.48)
    ok = np.isfinite(prof)
    assert abs(rc_[ok][np.argmax(prof[ok])] - Rs) < 2.5 * cfg.dx
    assert rel_l1(interior(W)[0], interior(W64)[0]) < 1e-2


@pytest.mark.parametrize("table", ["z1", "z1_uneven"])
def test_mixed_cooling_on_reference_tables(gpu_lib, golden, table):
    """The FP32 cooling of the mixed step on the reference's Z1.0.dat table
    (nodes uniform in log T: a cell's segment is guessed from log10 T) and on
    the same table with every other node of its lower half dropped (uneven:
    the binary search), against the FP64 step, both with the exact
    integrator: a 24^3 clumpy medium (log T uniform over 1e3-1e8 K) for 5
    steps, in which most cells cool and many cross segments within a step."""
    T, logL = golden["z1_T"], -golden["z1_b"]
    if table == "z1_uneven":
        half = len(T) // 2
        keep = [q for q in range(len(T)) if q >= half or q % 2 == 0]
        T, logL = T[keep], logL[keep]
    cfg, U0 = problems.clumpy(24, seed=2)
    cfg = tlq.Config(**{**cfg.__dict__, "cool_T": T, "cool_logL": logL, "cooling": tlq.COOL_EXACT,
                        "cool_sub_frac": 2e-3})
    U64, W64, (t64, it64, _, rc64), s64 = run_gpu(cfg, U0, 5, precision=tlq.PREC_FP64)
    Um, Wm, (tm, itm, _, rcm), sm = run_gpu(cfg, U0, 5, precision=tlq.PREC_MIXED)
    assert rc64 == tlq.OK and rcm == tlq.OK and it64 == itm == 5
    U0i = interior(U0)
    p0 = (cfg.gamma - 1.0) * (U0i[4] - 0.5 * (U0i[1] ** 2 + U0i[2] ** 2 + U0i[3] ** 2) / U0i[0])
    changed = np.mean(np.abs(interior(W64)[4] / p0 - 1.0) > 1e-3)
    assert changed > 0.3  # the cooling acts on a large part of the medium
    assert rel_l1(interior(Wm)[0], interior(W64)[0]) <= 1e-6
    assert rel_l1(interior(Wm)[4], interior(W64)[4]) <= 1e-5
    assert abs(sm[4] - s64[4]) / abs(s64[4]) <= 1e-8
