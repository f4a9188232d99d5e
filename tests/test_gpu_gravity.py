"""Self-gravity on the GPU (tlq_gravity.cu) against the oracle's MultiGrid
(source/sources.f90:99-787).

With the serial build's boundary values (zero) every level of the GPU solver
runs the reference's smoother in its order with FP64 arithmetic as the
restatement evaluates it, so one MultiGrid call and whole steps with
self-gravity are bit-identical to the oracle.  With the multipole faces the
moments are sums over all cells in another order, and the angles' cosines
and sines come from algebra (z/r, the Chebyshev recurrence, square roots)
instead of the reference's acos, atan2, cos, sin and real powers, so the bar
is 1e-10 of the potential (one call) and 1e-10 relative L1 per conserved
variable after the steps (the step's bar)."""
import numpy as np
import pytest

from oracle.oracle import Oracle, Run
from tests.helpers import face_ghost_mask, interior, oracle_params, rel_l1
from tlaloque_gb300 import problems, tlq

pytestmark = pytest.mark.gpu


def one_call(cfg, U0, phi0, it):
    """(GPU phi, GPU cycles, oracle phi, oracle cycles) of one MultiGrid call."""
    U = U0.copy(order="F")
    with tlq.Context(cfg) as ctx:
        ctx.borders(U, 1)
        g = phi0.copy(order="F")
        gc = ctx.multigrid(U, g, it)
    o = phi0.copy(order="F")
    oc = Oracle(oracle_params(cfg)).multigrid(U, o, it)
    return g, gc, o, oc


@pytest.mark.parametrize("n", [8, 16, 32, 64, 128])
def test_multigrid_bit_exact_zero_faces(gpu_lib, n):
    """One call from phi = 0 and one from a perturbed potential, bit for bit:
    levels of 8 to 128 cells relax in the cooperative kernel that holds each
    plane in shared memory, levels of 4 cells and fewer in the one-block
    coarse kernel."""
    cfg, U0 = problems.gravitating_cloud(n, grav_bc=tlq.GBC_ZERO)
    g, gc, o, oc = one_call(cfg, U0, np.zeros(cfg.phi_shape, order="F"), 0)
    assert gc == oc and gc >= 2
    np.testing.assert_array_equal(g, o)
    rng = np.random.default_rng(n)
    start = o * (1.0 + 0.01 * rng.standard_normal(o.shape))
    start[0] = start[-1] = 0.0
    start[:, 0] = start[:, -1] = 0.0
    start[:, :, 0] = start[:, :, -1] = 0.0
    g, gc, o, oc = one_call(cfg, U0, start, 3)
    assert gc == oc
    np.testing.assert_array_equal(g, o)


def test_multigrid_bit_exact_256(gpu_lib):
    """A 256^3 mesh: its finest level relaxes in the 512-thread, two blocks
    per SM variant of the pipelined kernel (256 planes resident at once)."""
    cfg, U0 = problems.gravitating_cloud(256, grav_bc=tlq.GBC_ZERO)
    g, gc, o, oc = one_call(cfg, U0, np.zeros(cfg.phi_shape, order="F"), 0)
    assert gc == oc and gc >= 2
    np.testing.assert_array_equal(g, o)


@pytest.mark.parametrize("n", [32, 128])
def test_multigrid_per_half_sweep_path(gpu_lib, n, monkeypatch):
    """The relax without the pipelined cooperative kernel (one launch per
    half-sweep, the path for levels whose planes cannot all be resident)
    gives the same bits too."""
    monkeypatch.setenv("TLQ_MG_PIPELINE", "0")
    cfg, U0 = problems.gravitating_cloud(n, grav_bc=tlq.GBC_ZERO)
    g, gc, o, oc = one_call(cfg, U0, np.zeros(cfg.phi_shape, order="F"), 0)
    assert gc == oc
    np.testing.assert_array_equal(g, o)


@pytest.mark.parametrize("n", [32, 128])
def test_multigrid_global_plane_path(gpu_lib, n, monkeypatch):
    """The skewed cooperative relax that reads every plane from the level
    arrays (the kernel of 256-cell levels) on levels that otherwise hold
    their planes in shared memory: the same bits."""
    monkeypatch.setenv("TLQ_MG_PLANE", "0")
    cfg, U0 = problems.gravitating_cloud(n, grav_bc=tlq.GBC_ZERO)
    g, gc, o, oc = one_call(cfg, U0, np.zeros(cfg.phi_shape, order="F"), 0)
    assert gc == oc
    np.testing.assert_array_equal(g, o)


@pytest.mark.parametrize("n", [16, 64])
def test_multigrid_multipole_faces(gpu_lib, n):
    """Multipole faces (it % 10 == 0): within 1e-10 of the potential.  The
    moments are sums of n^3 terms of both signs whose corner cells weigh
    (r/r_face)^4 ~ 9 times a face cell's in the l = 4 sums, so even the
    oracle's sequential sums carry ~sqrt(n^3) 9 eps ~ 1e-12 of round-off
    (2e-12 apart at 64^3); 1e-10 keeps the step's 1e-10 L1 bar."""
    cfg, U0 = problems.gravitating_cloud(n)
    g, gc, o, oc = one_call(cfg, U0, np.zeros(cfg.phi_shape, order="F"), 10)
    assert gc == oc
    scale = np.abs(o).max()
    assert scale > 0.0 and np.abs(g - o).max() <= 1e-10 * scale
    assert np.all(g[0, 1:-1, 1:-1] != 0.0)  # the faces were imposed


def run_both(cfg, U0, nsteps):
    run = Run(oracle_params(cfg), U0)
    run.run(nsteps)
    U1 = U0.copy(order="F")
    with tlq.Context(cfg) as ctx:
        ctx.borders(U1, 1)
        ctx.upload(U1)
        for _ in range(nsteps):
            ctx.step()
        Ug, Wg = ctx.state()
        t, it, dt, rc = ctx.time()
    return run, Ug, (t, it, dt, rc)


@pytest.mark.parametrize("n", [16, 64])
def test_step_self_gravity_bit_exact(gpu_lib, n):
    """Whole steps of the gravitating cloud with the serial build's faces
    (two MultiGrid calls per step, the stages' PHIT = PHIP + PHI), with a
    point mass at the centre too: bit-identical to the oracle."""
    cfg, U0 = problems.gravitating_cloud(n, grav_bc=tlq.GBC_ZERO, mass_msun=50.0)
    run, Ug, (t, it, dt, rc) = run_both(cfg, U0, 6)
    assert rc == tlq.OK and it == 6
    m = face_ghost_mask(cfg)
    np.testing.assert_array_equal(Ug[:, m], run.U[:, m])
    assert t == run.t and dt == run.dt


def test_step_graph_loop_node(gpu_lib, monkeypatch):
    """The step's graph runs the V-cycles as the body of a while node (only
    the cycles the loop test asks for are launched); with TLQ_MG_GRAPH_LOOP=0
    it holds the fixed sequence of 31 cycle slots instead.  Both give the
    same bits over twelve steps across a multipole refresh."""
    cfg, U0 = problems.gravitating_cloud(32)
    out = []
    for loop in ("1", "0"):
        monkeypatch.setenv("TLQ_MG_GRAPH_LOOP", loop)
        U1 = U0.copy(order="F")
        with tlq.Context(cfg) as ctx:
            ctx.borders(U1, 1)
            ctx.upload(U1)
            ctx.advance(12)
            ctx.synchronize()
            Ug, _ = ctx.state()
            out.append((Ug, ctx.time()))
    (Ua, ta), (Ub, tb) = out
    assert ta[3] == tlq.OK and ta[1] == 12
    np.testing.assert_array_equal(Ua, Ub)
    assert ta == tb


def test_step_self_gravity_multipole(gpu_lib):
    """Twelve steps across a multipole refresh (it = 0 and 10): relative L1
    <= 1e-10 per conserved variable."""
    cfg, U0 = problems.gravitating_cloud(32)
    run, Ug, (t, it, dt, rc) = run_both(cfg, U0, 12)
    assert rc == tlq.OK and it == 12
    err = rel_l1(interior(Ug), interior(run.U))
    assert np.all(err <= 1e-10), err


def test_step_self_gravity_mixed(gpu_lib):
    """The mixed-precision step with self-gravity (FP64 potential, FP32
    source arithmetic) against the plain FP64 step after 10 steps: density
    and energy relative L1 <= 1e-6; the momenta start at zero (the cloud is
    at rest), so their L1 is small and FP32 round-off weighs more: <= 1e-5."""
    cfg, U0 = problems.gravitating_cloud(32)
    out = []
    for prec in (tlq.PREC_FP64, tlq.PREC_MIXED):
        c = tlq.Config(**{**cfg.__dict__, "precision": prec})
        U1 = U0.copy(order="F")
        with tlq.Context(c) as ctx:
            ctx.borders(U1, 1)
            ctx.upload(U1)
            ctx.advance(10)
            out.append(ctx.state()[0])
            assert ctx.time()[3] == tlq.OK
    err = rel_l1(interior(out[1]), interior(out[0]))
    assert err[0] <= 1e-6 and err[4] <= 1e-6 and np.all(err[1:4] <= 1e-5), err


def test_self_gravity_config_checks(gpu_lib):
    cfg, _ = problems.gravitating_cloud(16)
    for bad in (dict(nx=24, ny=24, nz=24), dict(nz=8), dict(bc=(tlq.BC_PERIODIC,) * 6), dict(grav_bc=5)):
        with pytest.raises(tlq.TlqError):
            tlq.Context(tlq.Config(**{**cfg.__dict__, **bad}))
    # periodic boundaries are fine with the serial build's (zero) faces
    with tlq.Context(tlq.Config(**{**cfg.__dict__, "bc": (tlq.BC_PERIODIC,) * 6, "grav_bc": tlq.GBC_ZERO})):
        pass


def test_multigrid_wait_runs_out(gpu_lib, monkeypatch):
    """Failure detection of the pipelined relax, without a fault: with the
    limit of its neighbour-progress polls set to 0 (TLQ_MG_WAIT_LIMIT when
    the context is created) a plane gives up at its first wait that is not
    already satisfied, sets the abort flag, and every block leaves the
    launch.  The calls return (nothing hangs) with TLQ_ERR_TIMEOUT -- the
    per-routine MultiGrid and a step, whose solves run inside its graph --
    and a context created afterwards with the default limit steps normally,
    bit-identical to the oracle."""
    cfg, U0 = problems.gravitating_cloud(32, grav_bc=tlq.GBC_ZERO)
    monkeypatch.setenv("TLQ_MG_WAIT_LIMIT", "0")
    U = U0.copy(order="F")
    with tlq.Context(cfg) as ctx:
        ctx.borders(U, 1)
        with pytest.raises(tlq.TlqError) as err:
            ctx.multigrid(U, np.zeros(cfg.phi_shape, order="F"), 0)
        assert err.value.code == tlq.ERR_TIMEOUT
        ctx.upload(U)
        with pytest.raises(tlq.TlqError) as err:
            ctx.step()
        assert err.value.code == tlq.ERR_TIMEOUT
    monkeypatch.delenv("TLQ_MG_WAIT_LIMIT")
    run = Run(oracle_params(cfg), U0)
    run.run(2)
    U = U0.copy(order="F")
    with tlq.Context(cfg) as ctx:
        ctx.borders(U, 1)
        ctx.upload(U)
        ctx.step()
        t, it, dt = ctx.step()
        Ug, _ = ctx.state()
    m = face_ghost_mask(cfg)
    assert (t, it, dt) == (run.t, run.it, run.dt)
    np.testing.assert_array_equal(Ug[:, m], run.U[:, m])
