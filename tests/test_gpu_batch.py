"""Batched persistent ensemble (tlq_batch_*): members of uneven sizes and
different physics advanced together must be bit for bit the same runs as
each member alone, whatever the z-chunking (every face goes through one copy
of the face code, and the dt reduction is a max); a failing member stops
alone; members stop at their own tfin; the autotuner's choice and cache, and
the state it restores."""
import json

import numpy as np
import pytest

from tests.helpers import interior
from tests.test_gpu_step import smooth_state
from tlaloque_gb300 import problems, tlq

pytestmark = pytest.mark.gpu


def mixed(cfg, **kw):
    return tlq.Config(**{**cfg.__dict__, "precision": tlq.PREC_MIXED, **kw})


def ensemble():
    """Four members: two wind bubbles of different sizes and winds, a Sedov
    blast, and a random field on a non-cubic periodic/reflective mesh."""
    a_cfg, a_U = problems.wind_bubble(32)
    b_cfg, b_U = problems.wind_bubble(48, vw_kms=900.0, n_amb=3.0)
    c_cfg, c_U = problems.sedov(40)
    d_cfg = tlq.Config(nx=33, ny=20, nz=24, xl=0.0, xr=1.0, yl=0.0, yr=0.6, zl=0.0, zr=0.7,
                       bc=(tlq.BC_REFLECTIVE, tlq.BC_OUTFLOW, tlq.BC_PERIODIC, tlq.BC_PERIODIC, tlq.BC_OUTFLOW,
                           tlq.BC_REFLECTIVE))
    d_U = smooth_state(d_cfg, seed=3, mach=1.1)
    return [(mixed(a_cfg), a_U), (mixed(b_cfg), b_U), (mixed(c_cfg), c_U), (mixed(d_cfg), d_U)]


def single(cfg, U0, nsteps, tfin=None):
    U1 = U0.copy(order="F")
    with tlq.Context(cfg) as ctx:
        ctx.borders(U1, 1)
        ctx.upload(U1)
        if tfin is not None:
            ctx.set_tfin(tfin)
        ctx.advance(nsteps)
        t, it, dt, rc = ctx.time()
        U, W = ctx.state()
    return U, (t, it, dt, rc)


def load(batch, members):
    for m, (cfg, U0) in zip(batch.members, members):
        U1 = U0.copy(order="F")
        m.borders(U1, 1)
        m.upload(U1)


def test_batch_matches_single_runs(gpu_lib):
    members = ensemble()
    n = 12
    with tlq.Batch([c for c, _ in members]) as b:
        load(b, members)
        b.run(n)
        assert b.status() == [tlq.OK] * 4
        got = [(m.state()[0], m.time()) for m in b.members]
        st = b.stats()
        assert st.members == 4 and st.graph == 1 and st.steps == n and st.items > 0
    for (cfg, U0), (U, tm) in zip(members, got):
        ref, tr = single(cfg, U0, n)
        assert tm[1] == tr[1] == n
        assert tm[0] == tr[0] and tm[2] == tr[2]
        np.testing.assert_array_equal(interior(U), interior(ref))


def rel_close(a, b, tol=1e-6):
    """FP32 round-off: max |a - b| per variable against that variable's scale."""
    for e in range(a.shape[0]):
        scale = np.max(np.abs(b[e])) + 1e-300
        assert np.max(np.abs(a[e] - b[e])) <= tol * scale, (e, np.max(np.abs(a[e] - b[e])) / scale)


def test_batch_tiling_does_not_change_results(gpu_lib):
    members = ensemble()
    outs = []
    for z in (8, 16):
        with tlq.Batch([c for c, _ in members]) as b:
            load(b, members)
            for i in range(len(members)):
                b.set_tiling(i, z)
            assert b.tiling() == [min(z, c.nz) for c, _ in members]
            b.run(6)
            outs.append([m.state()[0] for m in b.members])
    for u8, u16 in zip(*outs):
        np.testing.assert_array_equal(interior(u8), interior(u16))


def test_failing_member_is_isolated(gpu_lib):
    members = ensemble()
    cfg_bad, U_bad = members[3]
    U_bad = U_bad.copy(order="F")
    U_bad[0, 10, 10, 10] = -1.0  # a non-positive density: the member's dt / state go bad
    members[3] = (cfg_bad, U_bad)
    with tlq.Batch([c for c, _ in members]) as b:
        load(b, members)
        b.run(5)
        st = b.status()
        assert st[3] != tlq.OK
        assert st[:3] == [tlq.OK] * 3
        got = [m.state()[0] for m in b.members[:3]]
    for (cfg, U0), U in zip(members[:3], got):
        ref, _ = single(cfg, U0, 5)
        np.testing.assert_array_equal(interior(U), interior(ref))


def test_members_stop_at_their_own_tfin(gpu_lib):
    members = ensemble()[:2]
    _, (_, _, t0, _) = single(members[0][0], members[0][1], 1)  # member 0's first dt
    with tlq.Batch([c for c, _ in members]) as b:
        load(b, members)
        b.members[0].set_tfin(3.5 * t0)  # a few steps only
        b.run(10)
        t, it0, _, rc = b.members[0].time()
        _, it1, _, _ = b.members[1].time()
        U0b = b.members[0].state()[0]
    assert rc == tlq.OK and 1 <= it0 < 10 and it1 == 10
    ref, tr = single(members[0][0], members[0][1], 10, tfin=3.5 * t0)
    assert tr[1] == it0 and tr[0] == t
    np.testing.assert_array_equal(interior(U0b), interior(ref))


def test_autotune_chooses_restores_and_caches(gpu_lib, tmp_path):
    members = ensemble()
    cache = tmp_path / "tune.json"
    with tlq.Batch([c for c, _ in members]) as b:
        load(b, members)
        before = [m.state()[0] for m in b.members]
        t_before = [m.time() for m in b.members]
        chosen = b.autotune(str(cache), steps=2)
        assert all(z in (8, 16, 32, 64, 128) or z == c.nz for z, (c, _) in zip(chosen, members))
        after = [m.state()[0] for m in b.members]
        for u0, u1 in zip(before, after):
            np.testing.assert_array_equal(u0, u1)
        assert [m.time() for m in b.members] == t_before
        b.run(4)
        got = [m.state()[0] for m in b.members]
    doc = json.loads(cache.read_text())
    assert len(doc["tuned"]) == 4  # four distinct sizes
    for (cfg, U0), U in zip(members, got):
        ref, _ = single(cfg, U0, 4)
        np.testing.assert_array_equal(interior(U), interior(ref))
    # a second batch takes the cached choice without measuring
    with tlq.Batch([c for c, _ in members]) as b2:
        load(b2, members)
        assert b2.autotune(str(cache), steps=2) == chosen


@pytest.mark.parametrize("precision", [tlq.PREC_FP64, tlq.PREC_MIXED])
def test_context_autotune_restores_state(gpu_lib, tmp_path, precision):
    """Single-context tuner on the wind bubble (FP64: carried cooled pressure
    is state too): the run after tuning continues bit for bit (neither form
    depends on the tiling)."""
    cfg, U0 = problems.wind_bubble(40)
    cfg = tlq.Config(**{**cfg.__dict__, "precision": precision})
    ref, tr = single(cfg, U0, 6)
    cache = tmp_path / "tune1.json"
    U1 = U0.copy(order="F")
    with tlq.Context(cfg) as ctx:
        ctx.borders(U1, 1)
        ctx.upload(U1)
        ctx.advance(2)
        z = ctx.autotune(str(cache), steps=2)
        assert z == ctx.tiling() and z in (8, 16, 32, 40)
        ctx.advance(4)
        t, it, dt, rc = ctx.time()
        U = ctx.state()[0]
    assert rc == tlq.OK and it == 6
    np.testing.assert_array_equal(interior(U), interior(ref))
    assert t == tr[0]
    assert json.loads(cache.read_text())["tuned"]


def test_batch_with_surrogate_members(gpu_lib):
    """Members with the learned cooling surrogate (their three cooling passes
    join the captured batched step) advance exactly like their single runs;
    a plain member beside them is unaffected."""
    cfg_a, U_a = problems.wind_bubble(32)
    cfg_b, U_b = problems.clumpy(32, seed=5)
    exact = dict(cool_sub_frac=2e-3, cool_max_sub=20000)
    with tlq.Context(cfg_a) as tctx:
        tctx.train_cooling_surrogate(nsamples=1 << 20, epochs=4, seed=3)
        net = tctx.get_cooling_surrogate()
    members = [(mixed(cfg_a, cooling=tlq.COOL_MLP, **exact), U_a), (mixed(cfg_b, cooling=tlq.COOL_MLP, **exact), U_b),
               (mixed(cfg_b), U_b)]
    n = 6

    def single_mlp(cfg, U0):
        U1 = U0.copy(order="F")
        with tlq.Context(cfg) as ctx:
            if cfg.cooling == tlq.COOL_MLP:
                ctx.set_cooling_surrogate(*net)
            ctx.borders(U1, 1)
            ctx.upload(U1)
            ctx.advance(n)
            st = ctx.stats()
            return ctx.state()[0], ctx.time(), (st.cool_mlp, st.cool_fallback)

    with tlq.Batch([c for c, _ in members]) as b:
        for m, (cfg, _) in zip(b.members, members):
            if cfg.cooling == tlq.COOL_MLP:
                m.set_cooling_surrogate(*net)
        load(b, members)
        b.run(n)
        assert b.status() == [tlq.OK] * 3
        assert b.stats().launches_per_step == 2 + 3  # both surrogate members share the three cooling launches
        got = [(m.state()[0], m.time(), (m.stats().cool_mlp, m.stats().cool_fallback)) for m in b.members]
    for (cfg, U0), (U, tm, cc) in zip(members, got):
        ref, tr, rc = single_mlp(cfg, U0)
        assert tm == tr
        np.testing.assert_array_equal(interior(U), interior(ref))
        assert cc == rc
