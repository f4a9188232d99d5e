// tlq_noalloc.cu -- time_step (source/HydroCore.f90:113-155) for callers that
// cannot allocate device memory.
//
// Who needs this: a host whose device memory is owned by someone else -- an
// arena or pool allocator that has already reserved the GPU's memory (a
// further cudaMalloc can then fail, and it fragments the arena), or a
// time-critical step loop that cannot afford cudaMalloc/cudaFree's implicit
// device synchronisation.  Such callers hand in device buffers they already
// own; this entry point then allocates nothing at all: no cudaMalloc, no
// cudaFree, no allocating library routine.
//
// The ticket and the running maxima of the single-pass CFL reduction live in
// one file-scope device variable (below, 72 bytes), which every GPU that
// loads the library holds until the process exits.
#include "../../include/tlq.h"
#include "tlq_internal.h"

namespace tlq {
namespace {

constexpr int NA_THREADS = 256;
constexpr int NA_CELLS_PER_THREAD = 16;
constexpr long long NA_CELLS_PER_BLOCK = (long long)NA_THREADS * NA_CELLS_PER_THREAD;  // 4096

struct NoAllocScratch {
  Clock clk;  // the reduction's ticket and maxima (zero before a call) and its dt
};

// The scratch, per device.  Host code must not use this name as an address;
// it asks the runtime for the device address (below).
static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

// Same reduction as the per-routine time_step kernel, with a fixed chunk of
// NA_CELLS_PER_BLOCK interior cells per block.
__global__ void __launch_bounds__(NA_THREADS) k_time_step_noalloc(Params p, Aos A, const double* __restrict__ W,
                                                                  NoAllocScratch* sc, double* d_dt) {
  __shared__ double red[96];
  __shared__ int flag;
  const long long n = (long long)p.nx * p.ny * p.nz;
  const long long beg = (long long)blockIdx.x * NA_CELLS_PER_BLOCK;
  const long long end = beg + NA_CELLS_PER_BLOCK < n ? beg + NA_CELLS_PER_BLOCK : n;
  double m0 = 0.0, m1 = 0.0, m2 = 0.0;
  for (long long c = beg + threadIdx.x; c < end; c += NA_THREADS) {
    const int i = 1 + (int)(c % p.nx);
    const long long r = c / p.nx;
    const int j = 1 + (int)(r % p.ny);
    const int k = 1 + (int)(r / p.ny);
    const double* w = W + A.at(i, j, k);
    double ww[5], v3[3];
#pragma unroll
    for (int e = 0; e < 5; ++e) ww[e] = w[e];
    signal_speeds(p.gamma, ww, v3);
    m0 = max_nan(m0, v3[0]);
    m1 = max_nan(m1, v3[1]);
    m2 = max_nan(m2, v3[2]);
  }
  cfl_reduce_finalize<NA_THREADS>(m0, m1, m2, &sc->clk, p, false, red, &flag);
  if (flag && threadIdx.x == 0) *d_dt = sc->clk.dt;
}

// The device address of the scratch variable in the current context, looked
// up on every call (the lookup allocates nothing).  A cached address could
// outlive its module: after cudaDeviceReset the library's module is loaded
// again, and a caller that makes another driver context current sees another
// copy of the variable.  The first lookup in a context loads the module
// there; make that first call outside any stream capture.
cudaError_t scratch_address(NoAllocScratch** out) {
  void* ptr = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
  if (e != cudaSuccess) return e;
  *out = static_cast<NoAllocScratch*>(ptr);
  return cudaSuccess;
}

}  // namespace
}  // namespace tlq

extern "C" int tlq_time_step_noalloc(const double* d_uprim, int nx, int ny, int nz, double dx, double dy, double dz,
                                     double gamma, double cfl, double* d_dt, void* cuda_stream) {
  using namespace tlq;
  if (!d_uprim || !d_dt || nx < 1 || ny < 1 || nz < 1) return TLQ_ERR_ARG;
  const long long n = (long long)nx * ny * nz;
  NoAllocScratch* sc = nullptr;
  if (scratch_address(&sc) != cudaSuccess) return TLQ_ERR_CUDA;
  Params p{};
  p.nx = nx; p.ny = ny; p.nz = nz;
  p.dx = dx; p.dy = dy; p.dz = dz;
  p.gamma = gamma;
  p.cfl = cfl;
  const Aos A{nx, ny, nz};
  const long long nblk = (n + NA_CELLS_PER_BLOCK - 1) / NA_CELLS_PER_BLOCK;
  if (nblk > 0x7fffffffLL) return TLQ_ERR_ARG;  // beyond one grid's x extent
  const int nblocks = (int)nblk;
  cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
  // The scratch keeps the previous call's contents: ticket and maxima must start at 0.
  if (cudaMemsetAsync(&sc->clk, 0, sizeof(Clock), s) != cudaSuccess) return TLQ_ERR_CUDA;
  // The launch's own status (cudaGetLastError would also consume an error
  // left by the caller's earlier launches and report it as this call's).
  void* args[] = {&p, (void*)&A, (void*)&d_uprim, &sc, &d_dt};
  const cudaError_t e = cudaLaunchKernel((const void*)k_time_step_noalloc, dim3((unsigned)nblocks), dim3(NA_THREADS),
                                         args, 0, s);
  return e == cudaSuccess ? TLQ_OK : TLQ_ERR_CUDA;
}
