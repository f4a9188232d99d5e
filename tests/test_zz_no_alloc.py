"""tlq_time_step_noalloc: the time_step entry point for callers that cannot
allocate device memory (their GPU memory belongs to a pool or arena
allocator, or their step loop cannot take cudaMalloc's synchronisation).
Its input and output live in device buffers the caller already owns, and its
reduction scratch is one fixed variable inside the library.

Checked through the C ABI against the context-based tlq_time_step on the same
states, bit for bit (the tolerance of the per-routine tests), on two calls in
a row (the shared scratch must not leak the first call into the second).
This file sorts last so that a failing run that stops at the first failure
has already run every other test."""
import ctypes

import numpy as np
import pytest

from tlaloque_gb300 import problems, tlq

pytestmark = pytest.mark.gpu


def _bind(lib):
    f = lib.tlq_time_step_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                  ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p]
    return f


def test_time_step_noalloc_matches_time_step(gpu_lib):
    torch = pytest.importorskip("torch")
    f = _bind(gpu_lib)
    cfg = tlq.Config(nx=40, ny=36, nz=30, xl=0.0, xr=1.0, yl=0.0, yr=0.9, zl=0.0, zr=0.75, cfl=0.4)
    states = [problems.random_state(cfg, seed=21, mach=0.8), problems.random_state(cfg, seed=22, mach=2.5)]
    with tlq.Context(cfg) as ctx:
        Ws = [ctx.calc_prims(U) for U in states]
        want = [ctx.time_step(W) for W in Ws]
    assert want[0] != want[1]

    # Device buffers owned by the caller (here: allocated by torch).
    d_w = torch.empty(Ws[0].size, dtype=torch.float64, device="cuda")
    d_dt = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for W, ref in zip(Ws, want):
        d_w.copy_(torch.from_numpy(np.ravel(W, order="F")))
        torch.cuda.synchronize()
        rc = f(d_w.data_ptr(), cfg.nx, cfg.ny, cfg.nz, cfg.dx, cfg.dy, cfg.dz, cfg.gamma, cfg.cfl, d_dt.data_ptr(),
               stream)
        torch.cuda.synchronize()
        assert rc == tlq.OK
        assert d_dt.item() == ref


def test_time_step_noalloc_rejects_bad_arguments(gpu_lib):
    f = _bind(gpu_lib)
    dummy = ctypes.c_void_p(16)  # never dereferenced: the argument checks come first
    assert f(None, 8, 8, 8, 1.0, 1.0, 1.0, 5.0 / 3.0, 0.4, dummy, None) == tlq.ERR_ARG
    assert f(dummy, 8, 8, 8, 1.0, 1.0, 1.0, 5.0 / 3.0, 0.4, None, None) == tlq.ERR_ARG
    assert f(dummy, 0, 8, 8, 1.0, 1.0, 1.0, 5.0 / 3.0, 0.4, dummy, None) == tlq.ERR_ARG
    assert f(dummy, 8, -1, 8, 1.0, 1.0, 1.0, 5.0 / 3.0, 0.4, dummy, None) == tlq.ERR_ARG


def _uniform_with_hot_cell(torch, nx, ny, nz, cell):
    """UPrim (reference layout, on the device) of a uniform flow with one
    faster, hotter cell at interior cell (i, j, k) = cell."""
    W = torch.empty((nz + 4, ny + 4, nx + 4, 5), dtype=torch.float64, device="cuda")  # [k+1, j+1, i+1, var]
    W[...] = torch.tensor([1.0, 0.1, -0.2, 0.3, 1.0], dtype=torch.float64, device="cuda")
    i, j, k = cell
    W[k + 1, j + 1, i + 1] = torch.tensor([0.5, 3.0, -4.0, 5.0, 2.0], dtype=torch.float64, device="cuda")
    return W


def _block_cell(nx, ny, block):
    """Interior (i, j, k) of the first cell of reduction block `block`
    (4,096 interior cells per block, x fastest)."""
    c = 4096 * block
    return 1 + c % nx, 1 + (c // nx) % ny, 1 + c // (nx * ny)


def test_time_step_noalloc_large_mesh(gpu_lib):
    """A mesh of 330 x 330 x 310 cells (8,242 blocks of the reduction) with
    its one hot cell in the first, a middle and the last block: each dt is
    the one of a small mesh with the same two states, bit for bit (the
    maxima decide it), so the reduction keeps the maximum of whichever block
    holds it."""
    torch = pytest.importorskip("torch")
    f = _bind(gpu_lib)
    stream = torch.cuda.current_stream().cuda_stream
    spacing = (0.01, 0.012, 0.015)
    nx, ny, nz = 330, 330, 310
    nblocks = (nx * ny * nz + 4095) // 4096
    d_dt = torch.full((4,), -1.0, dtype=torch.float64, device="cuda")
    W = _uniform_with_hot_cell(torch, 8, 8, 8, (8, 7, 8))
    torch.cuda.synchronize()
    assert f(W.data_ptr(), 8, 8, 8, *spacing, 5.0 / 3.0, 0.4, d_dt[3:].data_ptr(), stream) == tlq.OK
    del W
    cells = [(1, 1, 1), _block_cell(nx, ny, 4000), (nx, ny - 1, nz)]
    assert (nx * ny * (cells[2][2] - 1) + nx * (cells[2][1] - 1) + cells[2][0] - 1) // 4096 == nblocks - 1
    for q, cell in enumerate(cells):
        W = _uniform_with_hot_cell(torch, nx, ny, nz, cell)
        torch.cuda.synchronize()
        rc = f(W.data_ptr(), nx, ny, nz, *spacing, 5.0 / 3.0, 0.4, d_dt[q:].data_ptr(), stream)
        torch.cuda.synchronize()
        assert rc == tlq.OK
        del W
    got = d_dt.tolist()
    assert got[3] > 0.0
    assert got[:3] == [got[3]] * 3


def test_time_step_noalloc_nonfinite_dt(gpu_lib):
    """A NaN in the state: tlq_time_step reports TLQ_ERR_NONFINITE_DT, the
    allocation-free entry point returns TLQ_OK (its status is known before
    the kernel runs) and writes the non-finite dt for the caller to check;
    the next call on a valid state is not affected."""
    torch = pytest.importorskip("torch")
    f = _bind(gpu_lib)
    cfg = tlq.Config(nx=16, ny=12, nz=10, xl=0.0, xr=1.0, yl=0.0, yr=0.75, zl=0.0, zr=0.625, cfl=0.4)
    U = problems.random_state(cfg, seed=5, mach=0.8)
    with tlq.Context(cfg) as ctx:
        W = ctx.calc_prims(U)
        want = ctx.time_step(W)
        Wbad = W.copy(order="F")
        Wbad[4, 7, 6, 5] = np.nan
        with pytest.raises(tlq.TlqError) as err:
            ctx.time_step(Wbad)
        assert err.value.code == tlq.ERR_NONFINITE_DT
    d_w = torch.empty(W.size, dtype=torch.float64, device="cuda")
    d_dt = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for state, check in ((Wbad, lambda dt: not np.isfinite(dt)), (W, lambda dt: dt == want)):
        d_w.copy_(torch.from_numpy(np.ravel(state, order="F")))
        torch.cuda.synchronize()
        rc = f(d_w.data_ptr(), cfg.nx, cfg.ny, cfg.nz, cfg.dx, cfg.dy, cfg.dz, cfg.gamma, cfg.cfl, d_dt.data_ptr(),
               stream)
        torch.cuda.synchronize()
        assert rc == tlq.OK
        assert check(d_dt.item())
