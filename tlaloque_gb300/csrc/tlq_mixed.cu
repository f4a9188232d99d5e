// tlq_mixed.cu -- the mixed-precision stage kernels (FP32 reconstruction,
// fluxes and sources; FP64 accumulation).  Built with --use_fast_math: FP32
// division and square root are the approximate hardware forms, FP32
// subnormals flush to zero; FP64 arithmetic is unaffected.
#include "tlq_internal.h"
#include "tlq_stage_mixed.cuh"

namespace tlq {

size_t mixed_smem_bytes() { return sizeof(MixedSmem); }

// The specialised instance: van Leer with HLLC, the reference's default
// pairing (user/parameters.f90); every other pairing runs the generic one.
constexpr int SPEC_LIM = LIM_VANLEER, SPEC_SOLV = SOLVER_HLLC;

cudaError_t prepare_mixed_kernels() {
  const int smem = (int)sizeof(MixedSmem);
  const void* ks[4] = {(const void*)stage_kernel_mixed<1>, (const void*)stage_kernel_mixed<2>,
                       (const void*)stage_kernel_mixed<1, SPEC_LIM, SPEC_SOLV>,
                       (const void*)stage_kernel_mixed<2, SPEC_LIM, SPEC_SOLV>};
  for (const void* k : ks) {
    const cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t launch_stage_mixed(int stage, const CUtensorMap& tm_in, const StageArgs& a, dim3 grid, cudaStream_t s) {
  const size_t smem = sizeof(MixedSmem);
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

}  // namespace tlq
