// tlq_probe.cu -- FP64 pipe throughput of the GPU the library runs on.
//
// The plain FP64 step is bound by the FP64 pipe, not by HBM; its roofline
// needs the rate of that pipe on this part, measured rather than quoted.
// Each thread runs independent dependency chains (enough of them, and enough
// blocks per SM, that the pipe and not the chain latency limits the rate)
// of one operation: an FMA (__fma_rn), an IEEE division (__ddiv_rn) or an
// IEEE square root (__dsqrt_rn), timed with CUDA events.  The operands keep
// every value finite and normal, so no special-case path is taken.
#include <cuda_runtime.h>

#include "../../include/tlq.h"

namespace tlq {
namespace {

constexpr int PR_THREADS = 256;
constexpr int PR_CHAINS = 8;

template <int OP>
__global__ void __launch_bounds__(PR_THREADS) k_fp64_rate(int iters, double seed, double* sink) {
  double x[PR_CHAINS];
#pragma unroll
  for (int c = 0; c < PR_CHAINS; ++c) x[c] = seed + 1e-3 * (threadIdx.x * PR_CHAINS + c);
  for (int n = 0; n < iters; ++n) {
#pragma unroll
    for (int c = 0; c < PR_CHAINS; ++c) {
      if (OP == 0) x[c] = __fma_rn(x[c], 0.9999999, 1e-7);  // fixed point near 1
      if (OP == 1) x[c] = __ddiv_rn(1.0000001, x[c]);      // oscillates near 1
      if (OP == 2) x[c] = __dsqrt_rn(x[c]) + 1e-9;         // converges to ~1
    }
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < PR_CHAINS; ++c) s += x[c];
  if (s == 12345.678) sink[threadIdx.x] = s;  // keeps the chains alive; never true
}

template <int OP>
cudaError_t time_op(int blocks, int iters, double* sink, cudaStream_t s, double* ops_per_s) {
  cudaEvent_t e0, e1;
  cudaError_t e = cudaEventCreate(&e0);
  if (e != cudaSuccess) return e;
  e = cudaEventCreate(&e1);
  if (e != cudaSuccess) {
    cudaEventDestroy(e0);
    return e;
  }
  k_fp64_rate<OP><<<blocks, PR_THREADS, 0, s>>>(iters / 8, 1.0, sink);  // warm-up
  cudaEventRecord(e0, s);
  k_fp64_rate<OP><<<blocks, PR_THREADS, 0, s>>>(iters, 1.0, sink);
  cudaEventRecord(e1, s);
  e = cudaEventSynchronize(e1);
  float ms = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  if (e == cudaSuccess) e = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (e != cudaSuccess) return e;
  *ops_per_s = (double)blocks * PR_THREADS * PR_CHAINS * (double)iters / (ms * 1e-3);
  return cudaSuccess;
}

}  // namespace
}  // namespace tlq

extern "C" int tlq_measure_fp64_rate(int device, double* fma_per_s, double* div_per_s, double* sqrt_per_s) {
  using namespace tlq;
  if (!fma_per_s || !div_per_s || !sqrt_per_s) return TLQ_ERR_ARG;
  int prev = 0;
  if (cudaGetDevice(&prev) != cudaSuccess || cudaSetDevice(device) != cudaSuccess) return TLQ_ERR_CUDA;
  int sms = 0;
  double* sink = nullptr;
  cudaStream_t s = nullptr;
  int rc = TLQ_OK;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
      cudaMalloc(&sink, PR_THREADS * sizeof(double)) != cudaSuccess ||
      cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) {
    rc = TLQ_ERR_CUDA;
  } else {
    const int blocks = sms * 8;
    if (time_op<0>(blocks, 4096, sink, s, fma_per_s) != cudaSuccess ||
        time_op<1>(blocks, 256, sink, s, div_per_s) != cudaSuccess ||
        time_op<2>(blocks, 256, sink, s, sqrt_per_s) != cudaSuccess)
      rc = TLQ_ERR_CUDA;
  }
  if (s) cudaStreamDestroy(s);
  if (sink) cudaFree(sink);
  cudaSetDevice(prev);
  return rc;
}
