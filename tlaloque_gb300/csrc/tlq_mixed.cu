// tlq_mixed.cu -- the mixed-precision stage kernels (FP32 reconstruction,
// fluxes and sources; FP64 accumulation).  Built with --use_fast_math: FP32
// division and square root are the approximate hardware forms, FP32
// subnormals flush to zero; FP64 arithmetic is unaffected.
#include "tlq_internal.h"
#include "tlq_stage_mixed.cuh"

namespace tlq {

size_t mixed_smem_bytes(int stage) { return stage == 1 ? sizeof(MixedSmem<1>) : sizeof(MixedSmem<2>); }

// The specialised instance: van Leer with HLLC, the reference's default
// pairing (user/parameters.f90); every other pairing runs the generic one.
constexpr int SPEC_LIM = LIM_VANLEER, SPEC_SOLV = SOLVER_HLLC;

cudaError_t prepare_mixed_kernels() {
  const void* ks[4] = {(const void*)stage_kernel_mixed<1>, (const void*)stage_kernel_mixed<2>,
                       (const void*)stage_kernel_mixed<1, SPEC_LIM, SPEC_SOLV>,
                       (const void*)stage_kernel_mixed<2, SPEC_LIM, SPEC_SOLV>};
  for (int q = 0; q < 4; ++q) {
    const int smem = (int)mixed_smem_bytes(q % 2 == 0 ? 1 : 2);
    const cudaError_t e = cudaFuncSetAttribute(ks[q], cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t launch_stage_mixed(int stage, const CUtensorMap& tm_in, const StageArgs& a, dim3 grid, cudaStream_t s) {
  const size_t smem = mixed_smem_bytes(stage);
  const bool spec = a.p.limiter == SPEC_LIM && a.p.solver == SPEC_SOLV;
  if (stage == 1) {
    if (spec)
      stage_kernel_mixed<1, SPEC_LIM, SPEC_SOLV><<<grid, MNT, smem, s>>>(tm_in, a);
    else
      stage_kernel_mixed<1><<<grid, MNT, smem, s>>>(tm_in, a);
  } else {
    if (spec)
      stage_kernel_mixed<2, SPEC_LIM, SPEC_SOLV><<<grid, MNT, smem, s>>>(tm_in, a);
    else
      stage_kernel_mixed<2><<<grid, MNT, smem, s>>>(tm_in, a);
  }
  return cudaGetLastError();
}

// calc_prims + time_step on an uploaded state (mainHD.f90:44,74) in the
// mixed form's arithmetic: FP32 primitives and signal speeds as stage 2 forms
// them for every later dt, the maxima and dt in FP64.  (The plain form's
// FP64 division and square root per cell take ~1.6 ms at 256^3 on the FP64
// pipe; this pass is bound by reading U.)
__global__ void __launch_bounds__(RED_THREADS) k_init_dt_mixed(Params p, Layout L, const double* __restrict__ U,
                                                               Clock* clk) {
  __shared__ double red[96];
  __shared__ int flag;
  const float gm1 = p.f_gamma - 1.0f, gf = p.f_gamma;
  const long long n = (long long)p.nx * p.ny * p.nz;
  float m0 = 0.0f, m1 = 0.0f, m2 = 0.0f;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    const int i = 1 + (int)(c % p.nx);
    const long long r = c / p.nx;
    const int j = 1 + (int)(r % p.ny);
    const int k = 1 + (int)(r / p.ny);
    const long long o = L.at(i, j, k);
    double u[5];
#pragma unroll
    for (int e = 0; e < 5; ++e) u[e] = U[e * L.plane + o];
    float cf[5], w[5];
    mixed_cell(gm1, u, 1, cf, w);
    const float cs = sqrtf(gf * w[4] / w[0]);
    const float v0 = fabsf(w[1]) + cs, v1 = fabsf(w[2]) + cs, v2 = fabsf(w[3]) + cs;
    m0 = (v0 != v0 || v0 > m0) ? v0 : m0;
    m1 = (v1 != v1 || v1 > m1) ? v1 : m1;
    m2 = (v2 != v2 || v2 > m2) ? v2 : m2;
  }
  cfl_reduce_finalize<RED_THREADS>(f2d(m0), f2d(m1), f2d(m2), clk, p, false, red, &flag);
}

cudaError_t launch_init_dt_mixed(const Params& p, const Layout& L, const double* U, Clock* clk, int nblocks,
                                 cudaStream_t s) {
  k_init_dt_mixed<<<nblocks, RED_THREADS, 0, s>>>(p, L, U, clk);
  return cudaGetLastError();
}

}  // namespace tlq
