// tlq_device.cuh -- device layout, clock, TMA/mbarrier helpers and the
// single-pass CFL grid reduction shared by the kernels of libtlq.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "tlq_physics.cuh"

namespace tlq {

// Status bits held in Clock::status (mapped to TLQ_ERR_* on the host).
constexpr int ST_NONFINITE_DT = 1;
constexpr int ST_NEG_DENSITY = 2;
constexpr int ST_TIMEOUT = 4;

// Device-resident time of the run (mainHD.f90's t, dt, it) and the state of
// the single-pass CFL reduction (its ticket and running maxima, zero between
// reductions).
struct Clock {
  double t;          // simulated time
  double dt;         // dt of the next step (time_step's result)
  double dt_used;    // dt of the last completed step
  double tfin;       // steps start only while t < tfin
  long long it;      // iterations
  unsigned int ticket;
  int status;
  unsigned long long vmax[3];  // max |u|+c, |v|+c, |w|+c so far, as max_key keys
};

// Structure-of-arrays mesh layout: 5 planes of px * nyg * nzg doubles (x
// fastest), cell (i, j, k) with i in -1..nx+2 at x index i+1.  px is a
// multiple of 8 so that every row starts on a 64-byte boundary.
struct Layout {
  int px, nyg, nzg;
  long long plane;
  __host__ __device__ __forceinline__ long long at(int i, int j, int k) const {
    return (long long)(i + 1) + (long long)px * ((long long)(j + 1) + (long long)nyg * (long long)(k + 1));
  }
};

// ---------------------------------------------------------------------------
// mbarrier / TMA helpers (inline PTX, sm_90+ forms valid on sm_103a).
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait: gives up after `limit` polls (each poll may suspend the
// thread for a short, hardware-chosen time).
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, long long limit) {
  for (long long n = 0; n < limit; ++n)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// 4-D tiled bulk tensor load global -> shared, completing on `bar`.
__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1, int c2,
                                            int c3) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(smem_u32(dst)),
      "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(bar))
      : "memory");
}

// Per-thread asynchronous copies global -> shared of one 8- or 4-byte
// value (cp.async), grouped by commit and awaited by the issuing thread.
__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_u32(dst)), "l"(__cvta_generic_to_global(src))
               : "memory");
}
__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32(dst)), "l"(__cvta_generic_to_global(src))
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// L1-bypassing load for values another block wrote in this launch.
__device__ __forceinline__ double ld_cg(const double* p) { return __ldcg(p); }

// ---------------------------------------------------------------------------
// Single-pass CFL reduction (time_step, source/HydroCore.f90:138-150):
// warp shuffles -> shared memory -> one maximum per block, folded into the
// clock's running maxima by 64-bit atomic max -> a ticket; the last block to
// arrive reads the three maxima and writes dt (and advances t, it when
// `advance` is set, as `step` does at HydroCore.f90:208-209).  No block ever
// waits for another, and the maximum is exact whatever the order.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double warp_max_nan(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = max_nan(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

template <int NTHREADS>
__device__ __forceinline__ void block_max3(double& a, double& b, double& c, double* red /*3*32*/) {
  a = warp_max_nan(a);
  b = warp_max_nan(b);
  c = warp_max_nan(c);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  constexpr int NW = NTHREADS / 32;
  __syncthreads();
  if (lane == 0) {
    red[warp] = a;
    red[32 + warp] = b;
    red[64 + warp] = c;
  }
  __syncthreads();
  if (warp == 0) {
    a = lane < NW ? red[lane] : 0.0;
    b = lane < NW ? red[32 + lane] : 0.0;
    c = lane < NW ? red[64 + lane] : 0.0;
    a = warp_max_nan(a);
    b = warp_max_nan(b);
    c = warp_max_nan(c);
  }
}

// A maximum of signal speeds as an unsigned key whose integer order is
// max_nan's order from 0: the bits of a positive double order like its value,
// a NaN takes the largest key (it wins, as max_nan lets it), and values <= 0
// the key 0 (they never beat the reduction's starting 0).  Key 0 reads back
// as +0.0 and the largest key as a NaN.
__device__ __forceinline__ unsigned long long max_key(double x) {
  if (x != x) return ~0ull;
  return x > 0.0 ? (unsigned long long)__double_as_longlong(x) : 0ull;
}
__device__ __forceinline__ double key_value(unsigned long long k) { return __longlong_as_double((long long)k); }

// Thread 0 folds a block's maxima (from block_max3) into the clock's.
__device__ __forceinline__ void cfl_fold(double a, double b, double c, Clock* clk) {
  atomicMax(&clk->vmax[0], max_key(a));
  atomicMax(&clk->vmax[1], max_key(b));
  atomicMax(&clk->vmax[2], max_key(c));
}

// A block's maxima without finishing the reduction (a later kernel of the
// same step, stream-ordered after this one, finishes it).
template <int NTHREADS>
__device__ __forceinline__ void cfl_contribute(double a, double b, double c, Clock* clk, double* red) {
  block_max3<NTHREADS>(a, b, c, red);
  if (threadIdx.x == 0) cfl_fold(a, b, c, clk);
}

// nblocks: the blocks (tiles) of this reduction, each arriving once (a
// persistent kernel reduces per mesh over the tiles it works through).
// Maxima that earlier kernels of the step folded in (cfl_contribute) take
// part.  *s_flag is set in the block that finished.
template <int NTHREADS>
__device__ void cfl_reduce_finalize_n(double a, double b, double c, Clock* clk, const Params& p, bool advance,
                                      double* red, int* s_flag, unsigned nblocks) {
  block_max3<NTHREADS>(a, b, c, red);
  if (threadIdx.x == 0) {
    cfl_fold(a, b, c, clk);
    __threadfence();
    const unsigned t = atomicAdd(&clk->ticket, 1u);
    *s_flag = (t == nblocks - 1);
  }
  __syncthreads();
  if (!*s_flag || threadIdx.x != 0) return;
  __threadfence();
  unsigned long long* vm = clk->vmax;
  const double m0 = key_value(__ldcg(vm)), m1 = key_value(__ldcg(vm + 1)), m2 = key_value(__ldcg(vm + 2));
  const double dtn = cfl_dt(p.cfl, p.dx, p.dy, p.dz, m0, m1, m2);
  if (advance) {
    clk->t = clk->t + clk->dt;
    clk->it = clk->it + 1;
    clk->dt_used = clk->dt;
  }
  clk->dt = dtn;
  if (!(dtn > 0.0) || dtn != dtn || dtn > 1.0e300) atomicOr(&clk->status, ST_NONFINITE_DT);
  vm[0] = vm[1] = vm[2] = 0ull;
  clk->ticket = 0u;
  __threadfence();
}

template <int NTHREADS>
__device__ __forceinline__ void cfl_reduce_finalize(double a, double b, double c, Clock* clk, const Params& p,
                                                    bool advance, double* red, int* s_flag) {
  cfl_reduce_finalize_n<NTHREADS>(a, b, c, clk, p, advance, red, s_flag, gridDim.x * gridDim.y * gridDim.z);
}

}  // namespace tlq
