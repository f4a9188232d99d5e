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


def _uniform_with_hot_cell(torch, nx, ny, nz):
    """UPrim (reference layout, on the device) of a uniform flow with one
    faster, hotter cell at interior (nx, ny - 1, nz), the last block's."""
    W = torch.empty((nz + 4, ny + 4, nx + 4, 5), dtype=torch.float64, device="cuda")  # [k+1, j+1, i+1, var]
    W[...] = torch.tensor([1.0, 0.1, -0.2, 0.3, 1.0], dtype=torch.float64, device="cuda")
    W[nz + 1, ny, nx + 1] = torch.tensor([0.5, 3.0, -4.0, 5.0, 2.0], dtype=torch.float64, device="cuda")
    return W


def test_time_step_noalloc_large_mesh(gpu_lib):
    """A mesh of 330 x 330 x 310 cells (8,242 blocks of the reduction): the
    dt is the one of a small mesh with the same two states, bit for bit
    (the maxima decide it), so every block's maximum reached the result."""
    torch = pytest.importorskip("torch")
    f = _bind(gpu_lib)
    d_dt = torch.full((2,), -1.0, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    spacing = (0.01, 0.012, 0.015)
    for q, (nx, ny, nz) in enumerate([(330, 330, 310), (8, 8, 8)]):
        W = _uniform_with_hot_cell(torch, nx, ny, nz)
        torch.cuda.synchronize()
        rc = f(W.data_ptr(), nx, ny, nz, *spacing, 5.0 / 3.0, 0.4, d_dt[q:].data_ptr(), stream)
        torch.cuda.synchronize()
        assert rc == tlq.OK
        del W
    big, small = d_dt.tolist()
    assert big > 0.0 and big == small
