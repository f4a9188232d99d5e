// tlq_kernels.cu -- FP64 kernels of libtlq: the fused stage kernels (plain
// FP64 instantiation), layout conversions, the initial prims + CFL pass, the
// potential, and the per-routine kernels on the reference layout.
//
// Built with -fmad=false: no multiply-add is contracted, so every result is
// bit-identical to the reference's FP64 arithmetic (transcendentals aside).
#include <algorithm>

#include "tlq_internal.h"
#include "tlq_convert.cuh"

namespace tlq {

namespace {
inline int div_up(long long a, long long b) { return (int)((a + b - 1) / b); }
constexpr int BT = 256;  // block size of the simple kernels
}  // namespace

// ===========================================================================
// Fused stage kernels
// ===========================================================================
size_t stage_smem_bytes(int /*precision*/) { return sizeof(StageSmem<double>); }

cudaError_t prepare_stage_kernels() {
  const int smem = (int)sizeof(StageSmem<double>);
  cudaError_t e = cudaFuncSetAttribute(stage_kernel<1, double>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(stage_kernel<2, double>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
}

cudaError_t launch_stage(int stage, int /*precision*/, const CUtensorMap& tm_in, const CUtensorMap& tm_p,
                         const StageArgs& a, dim3 grid, cudaStream_t s) {
  const size_t smem = sizeof(StageSmem<double>);
  if (stage == 1)
    stage_kernel<1, double><<<grid, NT, smem, s>>>(tm_in, tm_p, a);
  else
    stage_kernel<2, double><<<grid, NT, smem, s>>>(tm_in, tm_p, a);
  return cudaGetLastError();
}

// ===========================================================================
// Layout conversions (reference AoS <-> device SoA), all cells.  A block
// moves BT consecutive cells at a time through shared memory, so that the
// AoS side (5 * BT contiguous doubles, possibly a page-locked host array read
// or written over the host link) is touched with fully coalesced accesses and
// the SoA side with one coalesced access per variable.
// ===========================================================================
__device__ __forceinline__ long long soa_offset(const Aos& A, const Layout& L, long long c) {
  const int i = (int)(c % (A.nx + 4)) - 1;
  const long long r = c / (A.nx + 4);
  const int j = (int)(r % (A.ny + 4)) - 1;
  const int k = (int)(r / (A.ny + 4)) - 1;
  return L.at(i, j, k);
}

__global__ void __launch_bounds__(BT) k_aos_to_soa(Aos A, Layout L, const double* __restrict__ src,
                                                   double* __restrict__ dst) {
  __shared__ double sh[5 * BT];
  const long long n = A.cells();
  for (long long base = (long long)blockIdx.x * BT; base < n; base += (long long)gridDim.x * BT) {
    const int cnt = (int)min((long long)BT, n - base);
    for (int t = threadIdx.x; t < 5 * cnt; t += BT) sh[t] = src[5 * base + t];
    __syncthreads();
    if (threadIdx.x < cnt) {
      const long long o = soa_offset(A, L, base + threadIdx.x);
#pragma unroll
      for (int e = 0; e < 5; ++e) dst[e * L.plane + o] = sh[5 * threadIdx.x + e];
    }
    __syncthreads();
  }
}

__global__ void __launch_bounds__(BT) k_soa_to_aos(Aos A, Layout L, const double* __restrict__ src,
                                                   double* __restrict__ dst) {
  __shared__ double sh[5 * BT];
  const long long n = A.cells();
  for (long long base = (long long)blockIdx.x * BT; base < n; base += (long long)gridDim.x * BT) {
    const int cnt = (int)min((long long)BT, n - base);
    if (threadIdx.x < cnt) {
      const long long o = soa_offset(A, L, base + threadIdx.x);
#pragma unroll
      for (int e = 0; e < 5; ++e) sh[5 * threadIdx.x + e] = src[e * L.plane + o];
    }
    __syncthreads();
    for (int t = threadIdx.x; t < 5 * cnt; t += BT) dst[5 * base + t] = sh[t];
    __syncthreads();
  }
}

// UPrim for output: calc_prims of every cell, with the carried (cooled)
// pressure on the interior when P is given (apply_cooling updates UPrim(5)).
// With a clock, the state is U or U1 by the clock's buffer parity
// ((it - it_base) & 1), so that the kernel can be queued behind steps whose
// count the host does not know yet.
__global__ void __launch_bounds__(BT) k_prims_soa_to_aos(Params p, Aos A, Layout L, const double* U0,
                                                         const double* U1, const Clock* clk, long long it_base,
                                                         const double* __restrict__ P, double* __restrict__ W) {
  __shared__ double sh[5 * BT];
  const double* __restrict__ U = (clk && ((clk->it - it_base) & 1LL)) ? U1 : U0;
  const long long n = A.cells();
  for (long long base = (long long)blockIdx.x * BT; base < n; base += (long long)gridDim.x * BT) {
    const int cnt = (int)min((long long)BT, n - base);
    if (threadIdx.x < cnt) {
      const long long c = base + threadIdx.x;
      const int i = (int)(c % (A.nx + 4)) - 1;
      const long long r = c / (A.nx + 4);
      const int j = (int)(r % (A.ny + 4)) - 1;
      const int k = (int)(r / (A.ny + 4)) - 1;
      const long long o = L.at(i, j, k);
      double u[5], w[5];
#pragma unroll
      for (int e = 0; e < 5; ++e) u[e] = U[e * L.plane + o];
      cons2prim(p.gamma, u, w);
      if (P && i >= 1 && i <= p.nx && j >= 1 && j <= p.ny && k >= 1 && k <= p.nz) w[4] = P[o];
#pragma unroll
      for (int e = 0; e < 5; ++e) sh[5 * threadIdx.x + e] = w[e];
    }
    __syncthreads();
    for (int t = threadIdx.x; t < 5 * cnt; t += BT) W[5 * base + t] = sh[t];
    __syncthreads();
  }
}

static int conv_blocks(const Aos& A) {
  const long long n = A.cells();
  return (int)std::min<long long>((n + BT - 1) / BT, 152LL * 16);
}

cudaError_t launch_aos_to_soa(const Aos& A, const Layout& L, const double* src, double* dst, cudaStream_t s) {
  k_aos_to_soa<<<conv_blocks(A), BT, 0, s>>>(A, L, src, dst);
  return cudaGetLastError();
}
cudaError_t launch_soa_to_aos(const Aos& A, const Layout& L, const double* src, double* dst, cudaStream_t s) {
  k_soa_to_aos<<<conv_blocks(A), BT, 0, s>>>(A, L, src, dst);
  return cudaGetLastError();
}
cudaError_t launch_prims_soa_to_aos(const Params& p, const Aos& A, const Layout& L, const double* U, const double* P,
                                    double* W, cudaStream_t s) {
  k_prims_soa_to_aos<<<conv_blocks(A), BT, 0, s>>>(p, A, L, U, U, nullptr, 0, P, W);
  return cudaGetLastError();
}
cudaError_t launch_prims_soa_to_aos_clocked(const Params& p, const Aos& A, const Layout& L, const double* U0,
                                            const double* U1, const Clock* clk, long long it_base, const double* P,
                                            double* W, cudaStream_t s) {
  k_prims_soa_to_aos<<<conv_blocks(A), BT, 0, s>>>(p, A, L, U0, U1, clk, it_base, P, W);
  return cudaGetLastError();
}

// ===========================================================================
// Initial calc_prims + time_step over the interior of the uploaded state
// (mainHD.f90:44 and the first :74).  Grid-stride, single-pass reduction.
// ===========================================================================
int init_blocks(const Params& p) {
  const long long n = (long long)p.nx * p.ny * p.nz;
  return (int)std::max<long long>(1, std::min<long long>((n + RED_THREADS - 1) / RED_THREADS, 152LL * 8));
}

__global__ void __launch_bounds__(RED_THREADS) k_init_prims_dt(Params p, Layout L, const double* __restrict__ U,
                                                               double* __restrict__ P, Clock* clk) {
  __shared__ double red[96];
  __shared__ int flag;
  const long long n = (long long)p.nx * p.ny * p.nz;
  double m0 = 0.0, m1 = 0.0, m2 = 0.0;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    const int i = 1 + (int)(c % p.nx);
    const long long r = c / p.nx;
    const int j = 1 + (int)(r % p.ny);
    const int k = 1 + (int)(r / p.ny);
    const long long o = L.at(i, j, k);
    double u[5], w[5], v3[3];
#pragma unroll
    for (int e = 0; e < 5; ++e) u[e] = U[e * L.plane + o];
    cons2prim(p.gamma, u, w);
    if (P) P[o] = w[4];
    signal_speeds(p.gamma, w, v3);
    m0 = max_nan(m0, v3[0]);
    m1 = max_nan(m1, v3[1]);
    m2 = max_nan(m2, v3[2]);
  }
  cfl_reduce_finalize<RED_THREADS>(m0, m1, m2, clk, p, false, red, &flag);
}

cudaError_t launch_init_prims_dt(const Params& p, const Layout& L, const double* U, double* P, Clock* clk,
                                 int nblocks, cudaStream_t s) {
  k_init_prims_dt<<<nblocks, RED_THREADS, 0, s>>>(p, L, U, P, clk);
  return cudaGetLastError();
}

// Global interior sums of the 5 conserved variables (deterministic: fixed
// per-block partials, then one block sums them in order).
__global__ void __launch_bounds__(RED_THREADS) k_sums_partial(Params p, Layout L, const double* __restrict__ U,
                                                              double* partials) {
  __shared__ double sh[5][RED_THREADS];
  const long long n = (long long)p.nx * p.ny * p.nz;
  double acc[5] = {0, 0, 0, 0, 0};
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    const int i = 1 + (int)(c % p.nx);
    const long long r = c / p.nx;
    const int j = 1 + (int)(r % p.ny);
    const int k = 1 + (int)(r / p.ny);
    const long long o = L.at(i, j, k);
#pragma unroll
    for (int e = 0; e < 5; ++e) acc[e] += U[e * L.plane + o];
  }
#pragma unroll
  for (int e = 0; e < 5; ++e) sh[e][threadIdx.x] = acc[e];
  __syncthreads();
  for (int st = RED_THREADS / 2; st > 0; st >>= 1) {
    if ((int)threadIdx.x < st)
#pragma unroll
      for (int e = 0; e < 5; ++e) sh[e][threadIdx.x] += sh[e][threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x < 5) partials[5 * blockIdx.x + threadIdx.x] = sh[threadIdx.x][0];
}

__global__ void k_sums_final(const double* partials, int nblocks, double* out5) {
  if (threadIdx.x < 5) {
    double a = 0.0;
    for (int b = 0; b < nblocks; ++b) a += partials[5 * b + threadIdx.x];
    out5[threadIdx.x] = a;
  }
}

cudaError_t launch_conserved_sums(const Params& p, const Layout& L, const double* U, double* partials, int nblocks,
                                  double* out5, cudaStream_t s) {
  k_sums_partial<<<nblocks, RED_THREADS, 0, s>>>(p, L, U, partials);
  k_sums_final<<<1, 32, 0, s>>>(partials, nblocks, out5);
  return cudaGetLastError();
}

__global__ void k_log10_inplace(double* v, int n) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n) v[q] = log10(v[q]);
}

cudaError_t launch_log10_inplace(double* v, int n, cudaStream_t s) {
  k_log10_inplace<<<div_up(n, BT), BT, 0, s>>>(v, n);
  return cudaGetLastError();
}

// ===========================================================================
// pointmass_potential, source/pointsource_gravity.f90:12-39 (phi starts at 0).
// ===========================================================================
__device__ __forceinline__ double point_phi(const Params& p, const double* xyzm, int n, int i, int j, int k) {
  const double x = xcoord(p, i), y = ycoord(p, j), z = zcoord(p, k);
  double v = 0.0;
  for (int s = 0; s < n; ++s) {
    const double* m = xyzm + 4 * s;
    const double r = sqrt((m[0] - x) * (m[0] - x) + (m[1] - y) * (m[1] - y) + (m[2] - z) * (m[2] - z));
    v = v - GR * m[3] / r;
  }
  return v;
}

__global__ void k_point_potential_soa(Params p, Layout L, const double* xyzm, int n, double* phi) {
  const long long tot = (long long)(p.nx + 2) * (p.ny + 2) * (p.nz + 2);
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < tot; c += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(c % (p.nx + 2));
    const long long r = c / (p.nx + 2);
    const int j = (int)(r % (p.ny + 2));
    const int k = (int)(r / (p.ny + 2));
    phi[L.at(i, j, k)] = point_phi(p, xyzm, n, i, j, k);
  }
}

__global__ void k_point_potential_ref(Params p, const double* xyzm, int n, double* phi) {
  const PhiLayout P{p.nx, p.ny, p.nz};
  const long long tot = (long long)(p.nx + 2) * (p.ny + 2) * (p.nz + 2);
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < tot; c += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(c % (p.nx + 2));
    const long long r = c / (p.nx + 2);
    const int j = (int)(r % (p.ny + 2));
    const int k = (int)(r / (p.ny + 2));
    // phi(i,j,k) = phi(i,j,k) - G M / r, accumulated onto the caller's phi.
    const double x = xcoord(p, i), y = ycoord(p, j), z = zcoord(p, k);
    double v = phi[P.at(i, j, k)];
    for (int s = 0; s < n; ++s) {
      const double* m = xyzm + 4 * s;
      const double rr = sqrt((m[0] - x) * (m[0] - x) + (m[1] - y) * (m[1] - y) + (m[2] - z) * (m[2] - z));
      v = v - GR * m[3] / rr;
    }
    phi[P.at(i, j, k)] = v;
  }
}

namespace {
__global__ void k_to_f32(const double* __restrict__ src, float* __restrict__ dst, long long n) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x)
    dst[q] = d2f(src[q]);
}
}  // namespace

cudaError_t launch_to_f32(const double* src, float* dst, long long n, cudaStream_t s) {
  k_to_f32<<<(unsigned)std::min<long long>((n + 255) / 256, 152 * 16), 256, 0, s>>>(src, dst, n);
  return cudaGetLastError();
}

cudaError_t launch_point_potential_soa(const Params& p, const Layout& L, const double* xyzm, int n, double* phi,
                                       cudaStream_t s) {
  const long long tot = (long long)(p.nx + 2) * (p.ny + 2) * (p.nz + 2);
  k_point_potential_soa<<<div_up(tot, BT), BT, 0, s>>>(p, L, xyzm, n, phi);
  return cudaGetLastError();
}
cudaError_t launch_point_potential_ref(const Params& p, const double* xyzm, int n, double* phi, cudaStream_t s) {
  const long long tot = (long long)(p.nx + 2) * (p.ny + 2) * (p.nz + 2);
  k_point_potential_ref<<<div_up(tot, BT), BT, 0, s>>>(p, xyzm, n, phi);
  return cudaGetLastError();
}

// ===========================================================================
// Per-routine kernels on the reference layout (one thread per cell / face).
// ===========================================================================
__device__ __forceinline__ void cell_of(long long c, int nxr, int nyr, int off, int& i, int& j, int& k) {
  i = (int)(c % nxr) + off;
  const long long r = c / nxr;
  j = (int)(r % nyr) + off;
  k = (int)(r / nyr) + off;
}

// calc_prims, source/HydroCore.f90:1-33 (all cells).
__global__ void k_calc_prims_aos(Params p, Aos A, double* __restrict__ W, const double* __restrict__ U) {
  const long long n = A.cells();
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    double u[5], w[5];
#pragma unroll
    for (int e = 0; e < 5; ++e) u[e] = U[5 * c + e];
    cons2prim(p.gamma, u, w);
#pragma unroll
    for (int e = 0; e < 5; ++e) W[5 * c + e] = w[e];
  }
}

// time_step, source/HydroCore.f90:113-155 (interior, single-pass reduction).
__global__ void __launch_bounds__(RED_THREADS) k_time_step_aos(Params p, Aos A, const double* __restrict__ W,
                                                               Clock* clk) {
  __shared__ double red[96];
  __shared__ int flag;
  const long long n = (long long)p.nx * p.ny * p.nz;
  double m0 = 0.0, m1 = 0.0, m2 = 0.0;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    cell_of(c, p.nx, p.ny, 1, i, j, k);
    const double* w = W + A.at(i, j, k);
    double ww[5], v3[3];
#pragma unroll
    for (int e = 0; e < 5; ++e) ww[e] = w[e];
    signal_speeds(p.gamma, ww, v3);
    m0 = max_nan(m0, v3[0]);
    m1 = max_nan(m1, v3[1]);
    m2 = max_nan(m2, v3[2]);
  }
  cfl_reduce_finalize<RED_THREADS>(m0, m1, m2, clk, p, false, red, &flag);
}

// HLLCFluxes / HLLFluxes, faces i, j, k in 0..n (source/HLLC.f90:94-96, :223-225).
__global__ void k_fluxes_aos(Params p, Aos A, const double* __restrict__ U, const double* __restrict__ W,
                             double* __restrict__ F, double* __restrict__ G, double* __restrict__ H, int choice) {
  const long long n = (long long)(p.nx + 1) * (p.ny + 1) * (p.nz + 1);
  const long long st[3] = {5LL, 5LL * (p.nx + 4), 5LL * (p.nx + 4) * (p.ny + 4)};
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    cell_of(c, p.nx + 1, p.ny + 1, 0, i, j, k);
    const long long o = A.at(i, j, k);
    for (int d = 1; d <= 3; ++d) {
      const long long sd = st[d - 1];
      double wll[5], wl[5], wr[5], wrr[5], UL[5], UR[5], ff[5];
#pragma unroll
      for (int e = 0; e < 5; ++e) {
        wl[e] = W[o + e];
        wr[e] = W[o + sd + e];
        UL[e] = U[o + e];
        UR[e] = U[o + sd + e];
      }
      if (choice == 2) {
#pragma unroll
        for (int e = 0; e < 5; ++e) {
          wll[e] = W[o - sd + e];
          wrr[e] = W[o + 2 * sd + e];
        }
        limiter(wll, wl, wr, wrr, p.limiter);
      }
      double* out = (d == 1) ? F : (d == 2 ? G : H);
      if (riemann(p.solver, p.gamma, p.g1, ff, wl, wr, UL, UR, d)) {
#pragma unroll
        for (int e = 0; e < 5; ++e) out[o + e] = ff[e];
      }
    }
  }
}

// Godunov, source/HLLC.f90:25-58 (+ dt * S_Solver(W, phi) when phi is given).
__global__ void k_godunov_aos(Params p, Aos A, double* __restrict__ out, const double* __restrict__ UU,
                              const double* __restrict__ F, const double* __restrict__ G,
                              const double* __restrict__ H, const double* __restrict__ W,
                              const double* __restrict__ phi, double dt) {
  const long long n = (long long)p.nx * p.ny * p.nz;
  const double dtdx = dt / p.dx, dtdy = dt / p.dy, dtdz = dt / p.dz;
  const PhiLayout P{p.nx, p.ny, p.nz};
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    cell_of(c, p.nx, p.ny, 1, i, j, k);
    const long long o = A.at(i, j, k);
    const long long ox = A.at(i - 1, j, k), oy = A.at(i, j - 1, k), oz = A.at(i, j, k - 1);
    double sv[5] = {0, 0, 0, 0, 0};
    if (phi) {
      double w[5];
#pragma unroll
      for (int e = 0; e < 5; ++e) w[e] = W[o + e];
      gravity_cell(p, w, phi[P.at(i + 1, j, k)] - phi[P.at(i - 1, j, k)], phi[P.at(i, j + 1, k)] - phi[P.at(i, j - 1, k)],
                   phi[P.at(i, j, k + 1)] - phi[P.at(i, j, k - 1)], sv);
    }
#pragma unroll
    for (int e = 0; e < 5; ++e) {
      double v = UU[o + e] - dtdx * (F[o + e] - F[ox + e]) - dtdy * (G[o + e] - G[oy + e]) - dtdz * (H[o + e] - H[oz + e]);
      if (phi) v = v + dt * sv[e];
      out[o + e] = v;
    }
  }
}

// One face-plane fill of boundariesI/II (non-MPI branches), over the full
// extent of the other two axes (the reference assigns whole planes).
__global__ void k_bc_plane_aos(Params p, Aos A, double* U, int axis, int side, int layers) {
  const int n3[3] = {p.nx, p.ny, p.nz};
  const int ua = (axis == 0) ? 1 : 0, vb = (axis == 2) ? 1 : 2;
  const long long tot = (long long)(n3[ua] + 4) * (n3[vb] + 4);
  const int bc = p.bc[2 * axis + side];
  const int N = n3[axis];
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < tot; c += (long long)gridDim.x * blockDim.x) {
    const int a = (int)(c % (n3[ua] + 4)) - 1;
    const int b = (int)(c / (n3[ua] + 4)) - 1;
    int dst[2], src[2], nl = 0, flip = 0;
    if (layers == 1) {
      if (bc == BC_OUTFLOW || bc == BC_REFLECTIVE) {
        dst[0] = side ? N + 1 : 0; src[0] = side ? N : 1; nl = 1; flip = (bc == BC_REFLECTIVE);
      } else if (bc == BC_PERIODIC) {
        dst[0] = side ? N + 1 : 0; src[0] = side ? 1 : N; nl = 1;
      }
    } else {
      if (bc == BC_OUTFLOW) {
        dst[0] = side ? N + 1 : 0; dst[1] = side ? N + 2 : -1; src[0] = src[1] = side ? N : 1; nl = 2;
      } else if (bc == BC_REFLECTIVE) {
        dst[0] = side ? N + 1 : 0; src[0] = side ? N : 1;
        dst[1] = side ? N + 2 : -1; src[1] = side ? N - 1 : 2; nl = 2; flip = 1;
      } else if (bc == BC_PERIODIC) {
        dst[0] = side ? N + 1 : -1; src[0] = side ? 1 : N - 1;
        dst[1] = side ? N + 2 : 0; src[1] = side ? 2 : N; nl = 2;
      }
    }
    double v[2][5];
    for (int l = 0; l < nl; ++l) {  // read every source before writing (array assignment)
      int s3[3];
      s3[axis] = src[l]; s3[ua] = a; s3[vb] = b;
      const long long o = A.at(s3[0], s3[1], s3[2]);
#pragma unroll
      for (int e = 0; e < 5; ++e) v[l][e] = (flip && e == axis + 1) ? -U[o + e] : U[o + e];
    }
    for (int l = 0; l < nl; ++l) {
      int d3[3];
      d3[axis] = dst[l]; d3[ua] = a; d3[vb] = b;
      const long long o = A.at(d3[0], d3[1], d3[2]);
#pragma unroll
      for (int e = 0; e < 5; ++e) U[o + e] = v[l][e];
    }
  }
}

__global__ void k_winds_aos(Params p, Aos A, double* U) {
  const long long n = A.cells();
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    cell_of(c, p.nx + 4, p.ny + 4, -1, i, j, k);
    double u[5];
#pragma unroll
    for (int e = 0; e < 5; ++e) u[e] = U[5 * c + e];
    bool hit = false;
    for (int s = 0; s < p.nwinds; ++s) hit |= wind_cell(p, p.winds[s], i, j, k, u);
    for (int s = 0; s < p.nplanes; ++s)
      if (k >= p.nz) {
        plane_wind_cell(p, p.planes[s], k, u);
        hit = true;
      }
    if (hit)
#pragma unroll
      for (int e = 0; e < 5; ++e) U[5 * c + e] = u[e];
  }
}

// step, source/HydroCore.f90:182-206 (Uold is a copy of U before the call).
__global__ void k_viscous_step_aos(Params p, Aos A, double* __restrict__ U, const double* __restrict__ UP,
                                   const double* __restrict__ Uold) {
  const long long n = A.cells();
  const long long sx = 5, sy = 5LL * (p.nx + 4), sz = 5LL * (p.nx + 4) * (p.ny + 4);
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    cell_of(c, p.nx + 4, p.ny + 4, -1, i, j, k);
    const long long o = 5 * c;
    const bool inside = i >= 1 && i <= p.nx && j >= 1 && j <= p.ny && k >= 1 && k <= p.nz;
#pragma unroll
    for (int e = 0; e < 5; ++e) {
      if (inside) {
        const double* q = Uold + o + e;
        U[o + e] = UP[o + e] + p.eta * (q[sx] + q[-sx] + q[sy] + q[-sy] + q[sz] + q[-sz] - 6.0 * q[0]);
      } else {
        U[o + e] = UP[o + e];
      }
    }
  }
}

// apply_cooling, source/cooling.f90:47-119 (interior).
__global__ void k_cooling_aos(Params p, Aos A, double* __restrict__ W, double* __restrict__ U, double dt) {
  const long long n = (long long)p.nx * p.ny * p.nz;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    cell_of(c, p.nx, p.ny, 1, i, j, k);
    const long long o = A.at(i, j, k);
    double w[5];
#pragma unroll
    for (int e = 0; e < 5; ++e) w[e] = W[o + e];
    double u4 = U[o + 4];
    cool_cell(p, w, u4, dt);
    W[o + 4] = w[4];
    U[o + 4] = u4;
  }
}

// S_Solver, source/sources.f90:872-897.
__global__ void k_gravity_source_aos(Params p, Aos A, const double* __restrict__ W, const double* __restrict__ phi,
                                     double* __restrict__ S) {
  const long long n = A.cells();
  const PhiLayout P{p.nx, p.ny, p.nz};
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    cell_of(c, p.nx + 4, p.ny + 4, -1, i, j, k);
    const long long o = 5 * c;
    const bool inside = i >= 1 && i <= p.nx && j >= 1 && j <= p.ny && k >= 1 && k <= p.nz;
    double sv[5] = {0, 0, 0, 0, 0};
    if (inside) {
      double w[5];
#pragma unroll
      for (int e = 0; e < 5; ++e) w[e] = W[o + e];
      gravity_cell(p, w, phi[P.at(i + 1, j, k)] - phi[P.at(i - 1, j, k)], phi[P.at(i, j + 1, k)] - phi[P.at(i, j - 1, k)],
                   phi[P.at(i, j, k + 1)] - phi[P.at(i, j, k - 1)], sv);
    }
#pragma unroll
    for (int e = 0; e < 5; ++e) S[o + e] = sv[e];
  }
}

static int grid_for(long long n) { return (int)std::max<long long>(1, std::min<long long>((n + BT - 1) / BT, 152LL * 16)); }

cudaError_t launch_calc_prims_aos(const Params& p, const Aos& A, double* W, const double* U, cudaStream_t s) {
  k_calc_prims_aos<<<grid_for(A.cells()), BT, 0, s>>>(p, A, W, U);
  return cudaGetLastError();
}
cudaError_t launch_time_step_aos(const Params& p, const Aos& A, const double* W, Clock* clk, int nblocks,
                                 cudaStream_t s) {
  k_time_step_aos<<<nblocks, RED_THREADS, 0, s>>>(p, A, W, clk);
  return cudaGetLastError();
}
cudaError_t launch_fluxes_aos(const Params& p, const Aos& A, const double* U, const double* W, double* F, double* G,
                              double* H, int choice, cudaStream_t s) {
  const long long n = (long long)(p.nx + 1) * (p.ny + 1) * (p.nz + 1);
  k_fluxes_aos<<<grid_for(n), BT, 0, s>>>(p, A, U, W, F, G, H, choice);
  return cudaGetLastError();
}
cudaError_t launch_godunov_aos(const Params& p, const Aos& A, double* out, const double* UU, const double* F,
                               const double* G, const double* H, const double* W, const double* phi, double dt,
                               cudaStream_t s) {
  k_godunov_aos<<<grid_for((long long)p.nx * p.ny * p.nz), BT, 0, s>>>(p, A, out, UU, F, G, H, W, phi, dt);
  return cudaGetLastError();
}
cudaError_t launch_borders_aos(const Params& p, const Aos& A, double* U, int order, cudaStream_t s) {
  // boundariesI order: x-, x+, y+, y-, z+, z-; boundariesII: x-, x+, y-, y+, z-, z+.
  const int o1[6][2] = {{0, 0}, {0, 1}, {1, 1}, {1, 0}, {2, 1}, {2, 0}};
  const int o2[6][2] = {{0, 0}, {0, 1}, {1, 0}, {1, 1}, {2, 0}, {2, 1}};
  const int n3[3] = {p.nx, p.ny, p.nz};
  for (int q = 0; q < 6; ++q) {
    const int axis = order == 1 ? o1[q][0] : o2[q][0];
    const int side = order == 1 ? o1[q][1] : o2[q][1];
    const int ua = (axis == 0) ? 1 : 0, vb = (axis == 2) ? 1 : 2;
    const long long tot = (long long)(n3[ua] + 4) * (n3[vb] + 4);
    k_bc_plane_aos<<<grid_for(tot), BT, 0, s>>>(p, A, U, axis, side, order == 1 ? 1 : 2);
  }
  if (p.nwinds > 0) k_winds_aos<<<grid_for(A.cells()), BT, 0, s>>>(p, A, U);
  return cudaGetLastError();
}
cudaError_t launch_winds_aos(const Params& p, const Aos& A, double* U, cudaStream_t s) {
  if (p.nwinds > 0) k_winds_aos<<<grid_for(A.cells()), BT, 0, s>>>(p, A, U);
  return cudaGetLastError();
}
cudaError_t launch_viscous_step_aos(const Params& p, const Aos& A, double* U, const double* UP, const double* Uold,
                                    cudaStream_t s) {
  k_viscous_step_aos<<<grid_for(A.cells()), BT, 0, s>>>(p, A, U, UP, Uold);
  return cudaGetLastError();
}
cudaError_t launch_cooling_aos(const Params& p, const Aos& A, double* W, double* U, double dt, cudaStream_t s) {
  k_cooling_aos<<<grid_for((long long)p.nx * p.ny * p.nz), BT, 0, s>>>(p, A, W, U, dt);
  return cudaGetLastError();
}
cudaError_t launch_gravity_source_aos(const Params& p, const Aos& A, const double* W, const double* phi, double* S,
                                      cudaStream_t s) {
  k_gravity_source_aos<<<grid_for(A.cells()), BT, 0, s>>>(p, A, W, phi, S);
  return cudaGetLastError();
}

}  // namespace tlq
