// tlq_mixed.cu -- the mixed-precision stage kernels (FP32 reconstruction,
// fluxes and sources; FP64 accumulation).  Built with --use_fast_math: FP32
// division and square root are the approximate hardware forms, FP32
// subnormals flush to zero; FP64 arithmetic is unaffected.
#include "tlq_internal.h"
#include "tlq_stage_mixed.cuh"

namespace tlq {

size_t mixed_smem_bytes() { return sizeof(MixedSmem); }

cudaError_t prepare_mixed_kernels() {
  const int smem = (int)sizeof(MixedSmem);
  cudaError_t e = cudaFuncSetAttribute(stage_kernel_mixed<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(stage_kernel_mixed<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
}

cudaError_t launch_stage_mixed(int stage, const CUtensorMap& tm_in, const StageArgs& a, dim3 grid, cudaStream_t s) {
  const size_t smem = sizeof(MixedSmem);
  if (stage == 1)
    stage_kernel_mixed<1><<<grid, NT, smem, s>>>(tm_in, a);
  else
    stage_kernel_mixed<2><<<grid, NT, smem, s>>>(tm_in, a);
  return cudaGetLastError();
}

}  // namespace tlq
