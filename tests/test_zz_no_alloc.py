"""tlq_time_step_noalloc: the time_step entry point for callers that cannot
allocate device memory (their GPU memory belongs to a pool or arena
allocator, or their step loop cannot take cudaMalloc's synchronisation).
Its input and output live in device buffers the caller already owns, and its
reduction scratch is a fixed array inside the library.

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


def test_time_step_noalloc_rejects_meshes_beyond_its_scratch(gpu_lib):
    f = _bind(gpu_lib)
    dummy = ctypes.c_void_p(16)  # never dereferenced: the size check comes first
    assert f(dummy, 400, 400, 400, 1.0, 1.0, 1.0, 5.0 / 3.0, 0.4, dummy, None) == tlq.ERR_ARG
    assert f(None, 8, 8, 8, 1.0, 1.0, 1.0, 5.0 / 3.0, 0.4, dummy, None) == tlq.ERR_ARG
    assert f(dummy, 0, 8, 8, 1.0, 1.0, 1.0, 5.0 / 3.0, 0.4, dummy, None) == tlq.ERR_ARG
