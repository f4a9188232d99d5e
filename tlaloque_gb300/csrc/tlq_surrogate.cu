// tlq_surrogate.cu -- the learned cooling surrogate in the step (mixed form,
// TLQ_COOL_MLP) and its training driver.
//
// In the step, stage 2 cools the cells the exact integrator takes in one
// step and leaves the other cells that cool (temp >= the table's first
// temperature, cooling.f90:71) and the CFL reduction to three passes
// (k_cool_sort, k_cool_net, k_cool_dt): for a cell inside the training box
// the network predicts r with ln(T/T_new) = tau (1 + tau r) from
// (log10 n, log10 T, log10 tau); the prediction is accepted when
// |T_pred - T_ex| <= tol T, T_ex the exact integrator's temperature (the
// closed-form solution of dT/dt = -(gamma-1) n Lambda(T)/k_B for the
// piecewise power-law table, cool_exact_dropf); otherwise, and for a cell
// outside the box, the cell takes T_ex.
// Built with --use_fast_math (FP32 part of the mixed form).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <numeric>
#include <random>

#include "tlq_ctx.h"
#include "tlq_mlp.cuh"
#include "tlq_stage_mixed.cuh"
#include "tlq_umma.cuh"

namespace tlq {
namespace {

struct SurrogateArgs {
  const mlp::SmemWeights* img;  // the network's image (launch_pack_weights)
  float norm[6];        // centre, half-width per feature
  float box[6];         // training box (lo, hi per feature)
  unsigned long long* counts;
};

constexpr int CT = 128;      // threads per block of the network pass
constexpr int FT = 128;      // threads per block of the dt pass
constexpr int PB = 152 * 3;  // blocks of each pass (at most): one resident wave of the network pass

// Blocks of each cooling pass for a mesh: enough for its cells to cool at
// once (2048 cells a block), at most one wave.
int pass_blocks(const Params& p) {
  const long long n = (long long)p.nx * p.ny * p.nz;
  return (int)std::max<long long>(4, std::min<long long>((n + 2047) / 2048, PB));
}

__device__ __forceinline__ void speeds_max(const float* w, float gf, float& m0, float& m1, float& m2) {
  const float cs = sqrtf(gf * w[4] / w[0]);
  const float v0 = fabsf(w[1]) + cs, v1 = fabsf(w[2]) + cs, v2 = fabsf(w[3]) + cs;
  m0 = (v0 != v0 || v0 > m0) ? v0 : m0;
  m1 = (v1 != v1 || v1 > m1) ? v1 : m1;
  m2 = (v2 != v2 || v2 > m2) ? v2 : m2;
}

__device__ __forceinline__ long long interior_offset(const Params& p, const Layout& L, long long cidx) {
  const int i = 1 + (int)(cidx % p.nx);
  const long long r = cidx / p.nx;
  const int j = 1 + (int)(r % p.ny);
  const int k = 1 + (int)(r / p.ny);
  return L.at(i, j, k);
}

// Pass 1 (sort): stage 2 queued the interior cells that cool (temp >= the
// table's first temperature, cooling.f90:71) beyond a single step of the
// exact integrator (it cooled the cells whose tau is at most the
// integrator's single-step limit itself, with this pass's arithmetic).  A
// cell inside the training box goes to the network queue; a cell outside it
// takes the exact integrator here; a queued cell whose tau is at most the
// single-step limit after all takes the single exponential step here.
// Pass 2 (network): the network queue densely, 32 cells to a warp (a warp
// of the sort pass holds a few network cells at most, and its matrix tiles
// would run for all 32 rows): the prediction, accepted when the residual
// check against the exact integrator passes, else the exact integrator's
// temperature (which the check has just computed).
// Both passes fold the block maxima of the signal speeds of the cells they
// cooled into the clock's (stage 2 left out the cells it queued); pass 3
// finishes the dt reduction and empties the queues.
// The state the step just wrote: U1 or U0 by the clock's buffer parity (the
// clock has not advanced yet), so that one captured launch serves both
// parities.
__device__ __forceinline__ double* step_output(double* U0, double* U1, const Clock* clk, long long it_base) {
  return ((clk->it - it_base) & 1LL) ? U0 : U1;
}

// Everything one mesh's cooling passes need (a kernel argument for one
// mesh, a device array entry for a batch of them).
struct CoolJob {
  Params p;  // the run's parameters, cooling = the exact integrator (the fallback)
  Layout L;
  double* U0;
  double* U1;
  long long it_base;
  Clock* clk;
  SurrogateArgs sa;
  const unsigned* cqueue;  // cells stage 2 queued (they cool)
  unsigned* cqcount;
  unsigned* nqueue;  // cells for the network
  unsigned* nqcount;
  unsigned blk0, nblk;  // this mesh's blocks of each pass: [blk0, blk0 + nblk)
};

// The mesh block b of a pass works on: `one` for a single mesh (jobs null),
// else the job whose block range holds b (ranges ascending, back to back).
__device__ __forceinline__ const CoolJob* job_of_block(const CoolJob& one, const CoolJob* jobs, int njobs,
                                                      unsigned b) {
  if (!jobs) return &one;
  int lo = 0, hi = njobs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (jobs[mid].blk0 <= b) lo = mid; else hi = mid - 1;
  }
  return &jobs[lo];
}

// A block's copy of its job in shared memory (8-byte words): the passes read
// their arguments from there whichever path launched them.
static_assert(sizeof(CoolJob) % 8 == 0 && alignof(CoolJob) <= 16, "CoolJob copies as 8-byte words");
struct SmemJob {
  alignas(16) unsigned long long w[sizeof(CoolJob) / 8];
};
__device__ __forceinline__ const CoolJob& stage_job(SmemJob& s, const CoolJob* src) {
  const unsigned long long* from = reinterpret_cast<const unsigned long long*>(src);
  for (int q = threadIdx.x; q < (int)(sizeof(CoolJob) / 8); q += blockDim.x) s.w[q] = from[q];
  __syncthreads();
  return *reinterpret_cast<const CoolJob*>(s.w);
}

// The cooling quantities of a queued cell from its state u: primitives w,
// temperature T, whether it cools (need), and for one that does its
// tau = Lambda n^2 dt / E_th, the network's normalised features and whether
// they lie in the training box.  One definition for both passes.
struct CellCool {
  float w[5], T, tau, lam, feat[3];
  bool need, inbox;
};
__device__ __forceinline__ void cell_cool(const Params& p, const SurrogateArgs& sa, const double* u, float dtf,
                                          CellCool& c) {
  const float gm1 = p.f_gamma - 1.0f;
  float cf[5];
  mixed_cell(gm1, u, 1, cf, c.w);
  c.T = (c.w[4] / c.w[0]) * p.f_cT;
  c.need = cools_at(p, c.T, u);
  c.tau = 0.f;
  c.lam = 0.f;
  c.feat[0] = c.feat[1] = c.feat[2] = 0.f;
  c.inbox = false;
  if (c.need) {
    const float nd = c.w[0] * p.f_inv_muamu;
    const float eth = c.w[4] / gm1;
    c.lam = cool_coef_f(p.cool, c.T);
    c.tau = (c.lam * nd) * (nd / eth) * dtf;
    const float f0 = log10f(nd), f1 = log10f(c.T), f2 = log10f(c.tau);
    // inclusive, with 1e-4 dex of slack for the FP32 logarithms of cells on
    // a face of the box (e.g. a medium at the table's first temperature)
    constexpr float SL = 1e-4f;
    c.inbox = f0 >= sa.box[0] - SL && f0 <= sa.box[1] + SL && f1 >= sa.box[2] - SL && f1 <= sa.box[3] + SL &&
              f2 >= sa.box[4] - SL && f2 <= sa.box[5] + SL;
    c.feat[0] = (f0 - sa.norm[0]) / sa.norm[1];
    c.feat[1] = (f1 - sa.norm[2]) / sa.norm[3];
    c.feat[2] = (f2 - sa.norm[4]) / sa.norm[5];
  }
}

// Warp-aggregated append of cell index v to a queue.
__device__ __forceinline__ void warp_append(bool take, unsigned v, unsigned* queue, unsigned* count) {
  const unsigned qm = __ballot_sync(0xffffffffu, take);
  if (!qm) return;
  const int lane = threadIdx.x & 31;
  unsigned basei = 0;
  if (lane == 0) basei = atomicAdd(count, (unsigned)__popc(qm));
  basei = __shfl_sync(0xffffffffu, basei, 0);
  if (take) queue[basei + __popc(qm & ((1u << lane) - 1u))] = v;
}

// The counters of the three outcomes (network, fallback, single step).
__device__ __forceinline__ void add_counts(const SurrogateArgs& sa, unsigned long long used, unsigned long long fell,
                                           unsigned long long one) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    used += __shfl_xor_sync(0xffffffffu, used, off);
    fell += __shfl_xor_sync(0xffffffffu, fell, off);
    one += __shfl_xor_sync(0xffffffffu, one, off);
  }
  if ((threadIdx.x & 31) == 0) {
    if (used) atomicAdd(&sa.counts[0], used);
    if (fell) atomicAdd(&sa.counts[1], fell);
    if (one) atomicAdd(&sa.counts[2], one);
  }
}

__device__ void cool_sort_mesh(const CoolJob& j, double* red, unsigned nblocks, unsigned bid) {
  const Params& p = j.p;
  const Layout& L = j.L;
  const Clock* clk = j.clk;
  if (!(clk->t < clk->tfin)) return;  // the step did not run (mainHD.f90:61)
  const long long n = (long long)*j.cqcount;
  if ((long long)bid * CT >= n) return;  // no queued cell for this block: nothing to fold
  double* __restrict__ U = step_output(j.U0, j.U1, clk, j.it_base);
  const float gm1 = p.f_gamma - 1.0f, gf = p.f_gamma;
  const float dtf = d2f(clk->dt);
  float m0 = 0.f, m1 = 0.f, m2 = 0.f;
  unsigned long long fell = 0, one = 0;
  // warp-uniform trip count (the appends are warp-wide)
  for (long long base = (long long)bid * CT; base < n; base += (long long)nblocks * CT) {
    const long long q = base + threadIdx.x;
    const bool valid = q < n;
    long long o = 0;
    unsigned cidx = 0;
    double u[5] = {1.0, 0.0, 0.0, 0.0, 1.0};
    if (valid) {
      cidx = j.cqueue[q];
      o = interior_offset(p, L, cidx);
#pragma unroll
      for (int e = 0; e < 5; ++e) u[e] = U[e * L.plane + o];
    }
    CellCool c;
    cell_cool(p, j.sa, u, dtf, c);
    const bool need = valid && c.need;
    // tau at most the single-step limit: the exact integrator is a single
    // exponential step, and the network has nothing to gain; outside the
    // training box the exact integrator's closed form (p.cooling: COOL_EXACT)
    const bool single = need && !(c.tau > p.f_cool_sub_frac);
    const bool net = need && !single && c.inbox;
    const bool ext = need && !single && !c.inbox;
    if (single || ext) {
      cool_cell_f(p, p.f_cT, p.f_inv_muamu, gm1, c.w, u[4], dtf, u);
      U[4 * L.plane + o] = u[4];
      speeds_max(c.w, gf, m0, m1, m2);
    }
    warp_append(net, cidx, j.nqueue, j.nqcount);
    fell += ext ? 1 : 0;
    one += single ? 1 : 0;
  }
  add_counts(j.sa, 0, fell, one);
  cfl_contribute<CT>(f2d(m0), f2d(m1), f2d(m2), j.clk, red);
}

__device__ void cool_net_mesh(const CoolJob& j, umma::Smem& S, double* red, unsigned nblocks, unsigned bid) {
  const Params& p = j.p;
  const Layout& L = j.L;
  const Clock* clk = j.clk;
  const SurrogateArgs& sa = j.sa;
  if (!(clk->t < clk->tfin)) return;
  const long long n = (long long)*j.nqcount;
  if ((long long)bid * CT >= n) return;  // no network cell for this block: no weights, nothing to fold
  double* __restrict__ U = step_output(j.U0, j.U1, clk, j.it_base);
  umma::load_weights(sa.img, S);
  umma::setup(S);
  const CoolTable& tab = p.cool;
  const float gm1 = p.f_gamma - 1.0f, gf = p.f_gamma;
  const float dtf = d2f(clk->dt);
  float m0 = 0.f, m1 = 0.f, m2 = 0.f;
  unsigned long long used = 0, fell = 0;
  uint32_t phase = 0;
  bool tc = true;  // the tensor-core path is healthy (block-wide)
  // block-uniform trip count: one 128-row MMA tile per iteration
  for (long long base = (long long)bid * CT; base < n; base += (long long)nblocks * CT) {
    const long long q = base + threadIdx.x;
    const bool valid = q < n;
    long long o = 0;
    unsigned cidx = 0;
    double u[5] = {1.0, 0.0, 0.0, 0.0, 1.0};
    if (valid) {
      cidx = j.nqueue[q];
      o = interior_offset(p, L, cidx);
#pragma unroll
      for (int e = 0; e < 5; ++e) u[e] = U[e * L.plane + o];
    }
    CellCool c;
    cell_cool(p, sa, u, dtf, c);
    float y = 0.f;
    if (tc) tc = umma::forward(S, c.feat, y, phase);
    bool ok = false;
    if (valid) {
      const float T = c.T, tau = c.tau;
      // the exact integrator's change and the network's, T_new/T - 1 (the
      // network's r: ln(T_new/T) = -(tau + tau^2 r); clamped at the table's
      // first temperature, where cooling stops).  A cell whose cooling
      // reaches that temperature within the step (the exact change is the
      // floor's, T_0/T - 1) takes the exact integrator: training leaves those
      // pairs out, and the network's prediction, clamped at the floor, could
      // only err on one side.
      const float qfloor = __fsub_rn(tab.Tf[0] / T, 1.0f);
      const float qx = cool_exact_dropf(tab, T, c.lam, tau);
      const float qf = fmaxf(expm1f(-(1.0f + tau * y) * tau), qfloor);
      ok = tc && qx > qfloor && fabsf(qf - qx) <= p.f_mlp_tol;
      if (ok) {
        const float dp = __fmul_rn(c.w[4], qf);
        c.w[4] = __fadd_rn(c.w[4], dp);
        U[4 * L.plane + o] = u[4] + f2d(dp / gm1);
      } else {
        cool_cell_f(p, p.f_cT, p.f_inv_muamu, gm1, c.w, u[4], dtf, u);  // the exact integrator
        U[4 * L.plane + o] = u[4];
      }
      speeds_max(c.w, gf, m0, m1, m2);
    }
    used += ok ? 1 : 0;
    fell += (valid && !ok) ? 1 : 0;
  }
  if (!tc) {
    // an MMA wait ran out: the cells above took the exact integrator; the
    // step reports the timeout
    if (threadIdx.x == 0) atomicOr(&const_cast<Clock*>(clk)->status, ST_TIMEOUT);
    umma::drain(S, phase);
  }
  umma::teardown(S);
  add_counts(sa, used, fell, 0);
  cfl_contribute<CT>(f2d(m0), f2d(m1), f2d(m2), j.clk, red);
}

// The sort and network passes of one mesh (jobs null: `one`) or of njobs
// meshes, each on its own range of the grid's blocks.  One kernel, one call
// site each: the single-mesh and batched steps run the same instructions,
// so their FP32 results agree bit for bit.
__global__ void __launch_bounds__(CT) k_cool_sort(const __grid_constant__ CoolJob one,
                                                  const CoolJob* __restrict__ jobs, int njobs) {
  __shared__ double red[96];
  __shared__ SmemJob sj;
  const CoolJob& j = stage_job(sj, job_of_block(one, jobs, njobs, blockIdx.x));
  cool_sort_mesh(j, red, j.nblk, blockIdx.x - j.blk0);
}

__global__ void __launch_bounds__(CT, 3) k_cool_net(const __grid_constant__ CoolJob one,
                                                 const CoolJob* __restrict__ jobs, int njobs) {
  __shared__ umma::Smem S;
  __shared__ double red[96];
  __shared__ SmemJob sj;
  const CoolJob& j = stage_job(sj, job_of_block(one, jobs, njobs, blockIdx.x));
  cool_net_mesh(j, S, red, j.nblk, blockIdx.x - j.blk0);
}

__device__ void cool_dt_mesh(const CoolJob& j, double* red, int* flag, unsigned nblocks) {
  Clock* clk = j.clk;
  if (!(clk->t < clk->tfin)) return;
  cfl_reduce_finalize_n<FT>(0.0, 0.0, 0.0, clk, j.p, true, red, flag, nblocks);
  if (*flag && threadIdx.x == 0) {
    *j.cqcount = 0u;
    *j.nqcount = 0u;
  }
}

// Pass 3: the dt reduction over the block maxima of stage 2 and the two
// cooling passes (this pass's blocks only take their tickets); the last
// block of a mesh empties its queues.  One mesh (jobs null: `one`) or njobs
// meshes, as the other passes.
__global__ void __launch_bounds__(FT) k_cool_dt(const __grid_constant__ CoolJob one, const CoolJob* __restrict__ jobs,
                                                int njobs) {
  __shared__ double red[96];
  __shared__ int flag;
  __shared__ SmemJob sj;
  const CoolJob& j = stage_job(sj, job_of_block(one, jobs, njobs, blockIdx.x));
  cool_dt_mesh(j, red, &flag, j.nblk);
}

}  // namespace

size_t cool_job_bytes() { return sizeof(CoolJob); }

void fill_cool_job(void* dst, const Params& p, const Layout& L, double* U0, double* U1, long long it_base, Clock* clk,
                   const void* img, const float norm[6], const double box[6], unsigned long long* counts,
                   const unsigned* cqueue, unsigned* cqcount, unsigned* nqueue, unsigned* nqcount, int blk0,
                   int nblk) {
  CoolJob j{};
  j.p = p;
  j.p.cooling = COOL_EXACT;  // the fallback: the exact integrator (single step up to the run's cool_sub_frac)
  j.L = L;
  j.U0 = U0;
  j.U1 = U1;
  j.it_base = it_base;
  j.clk = clk;
  j.sa.img = static_cast<const mlp::SmemWeights*>(img);
  for (int q = 0; q < 6; ++q) {
    j.sa.norm[q] = norm[q];
    j.sa.box[q] = (float)box[q];
  }
  j.sa.counts = counts;
  j.cqueue = cqueue;
  j.cqcount = cqcount;
  j.nqueue = nqueue;
  j.nqcount = nqcount;
  j.blk0 = (unsigned)blk0;
  j.nblk = (unsigned)nblk;
  std::memcpy(dst, &j, sizeof j);
}

cudaError_t launch_cool_mlp_dt(const Params& p, const Layout& L, double* U0, double* U1, long long it_base,
                               Clock* clk, const void* img, const float norm[6], const double box[6],
                               unsigned long long* counts, const unsigned* cqueue, unsigned* cqcount,
                               unsigned* nqueue, unsigned* nqcount, cudaStream_t s) {
  const int nb = pass_blocks(p);
  CoolJob j;
  fill_cool_job(&j, p, L, U0, U1, it_base, clk, img, norm, box, counts, cqueue, cqcount, nqueue, nqcount, 0, nb);
  k_cool_sort<<<nb, CT, 0, s>>>(j, nullptr, 1);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_cool_net<<<nb, CT, 0, s>>>(j, nullptr, 1);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_cool_dt<<<nb, FT, 0, s>>>(j, nullptr, 1);
  return cudaGetLastError();
}

int cool_pass_blocks(const Params& p) { return pass_blocks(p); }

cudaError_t launch_cool_mlp_dt_batch(const void* jobs, int njobs, int nblocks, cudaStream_t s) {
  const CoolJob* d = static_cast<const CoolJob*>(jobs);
  const CoolJob none{};
  k_cool_sort<<<nblocks, CT, 0, s>>>(none, d, njobs);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_cool_net<<<nblocks, CT, 0, s>>>(none, d, njobs);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_cool_dt<<<nblocks, FT, 0, s>>>(none, d, njobs);
  return cudaGetLastError();
}


}  // namespace tlq

// ===========================================================================
// Host side
// ===========================================================================
namespace {

int sfail(tlq_ctx* c, int code, const std::string& m) {
  if (c) c->err = m;
  return code;
}

#define SCK(call)                                                                                  \
  do {                                                                                             \
    cudaError_t e_ = (call);                                                                       \
    if (e_ != cudaSuccess) return sfail(ctx, TLQ_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// Parameters of the training pairs' integrator (the context's physics and
// table): the exact integrator's closed form when sub_frac is 0, else the
// sub-cycled integrator with the given sub-steps (extrapolated).
Params exact_params(const tlq_ctx* ctx, double sub_frac, int max_sub) {
  Params p = ctx->P;
  p.cooling = sub_frac > 0.0 ? COOL_SUBCYCLE : COOL_EXACT;
  p.cool_sub_frac = sub_frac;
  p.cool_max_sub = max_sub;
  return p;
}

// Initial parameters: uniform(-a, a) with a = sqrt(6/(fan_in + fan_out)).
void init_params(std::vector<float>& P, unsigned long long seed) {
  using namespace tlq::mlp;
  std::mt19937_64 rng(seed ^ 0x5eedULL);
  auto fill = [&](int off, int fo, int fi) {
    const float a = std::sqrt(6.0f / (float)(fi + fo));
    std::uniform_real_distribution<float> d(-a, a);
    for (int q = 0; q < fo * fi; ++q) P[off + q] = d(rng);
  };
  std::fill(P.begin(), P.end(), 0.0f);
  fill(OFF_W1, HID, IN);
  fill(OFF_W2, HID, HID);
  fill(OFF_W3, HID, HID);
  fill(OFF_W4, 1, HID);
  P[OFF_B4] = 0.0f;
}

}  // namespace

extern "C" {

void tlq_surrogate_opts_default(tlq_surrogate_opts* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->nsamples = 20000000LL;
  o->epochs = 30;
  o->batch = 4096;
  o->lr = 3e-3f;
  o->seed = 12345ULL;
  const double box[6] = {-4.0, 4.0, 4.0, 8.5, -8.0, 1.0};
  for (int q = 0; q < 6; ++q) o->box[q] = box[q];
  o->sub_frac = 0.0;  // the exact integrator's closed form
  o->max_sub = 20000;
}

int tlq_cooling_pairs(tlq_ctx* ctx, long long n, unsigned long long seed, const double* box6, double sub_frac,
                      int max_sub, float* X, float* Y, double* raw) {
  if (!ctx || n <= 0 || !box6 || !X || !Y || !(sub_frac >= 0.0) || max_sub < 1) return TLQ_ERR_ARG;
  if (!ctx->dT) return sfail(ctx, TLQ_ERR_STATE, "cooling table not set");
  float *dX = nullptr, *dY = nullptr;
  double* dR = nullptr;
  SCK(cudaMalloc(&dX, 3 * n * sizeof(float)));
  SCK(cudaMalloc(&dY, n * sizeof(float)));
  if (raw) SCK(cudaMalloc(&dR, 4 * n * sizeof(double)));
  const Params p = exact_params(ctx, sub_frac, max_sub);
  cudaError_t e = launch_cool_pairs(p, n, seed, box6, dX, dY, nullptr, dR, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(X, dX, 3 * n * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(Y, dY, n * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess && raw) e = cudaMemcpyAsync(raw, dR, 4 * n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  cudaFree(dX);
  cudaFree(dY);
  cudaFree(dR);
  if (e != cudaSuccess) return sfail(ctx, TLQ_ERR_CUDA, std::string("cooling pairs: ") + cudaGetErrorString(e));
  return TLQ_OK;
}

int tlq_train_cooling_surrogate(tlq_ctx* ctx, const tlq_surrogate_opts* opts, tlq_surrogate_report* rep) {
  using namespace tlq::mlp;
  if (!ctx) return TLQ_ERR_ARG;
  tlq_surrogate_opts o;
  if (opts) o = *opts; else tlq_surrogate_opts_default(&o);
  if (o.nsamples < 2 * o.batch || o.batch < 16 || o.epochs < 1) return sfail(ctx, TLQ_ERR_ARG, "bad training options");
  if (!ctx->dT) return sfail(ctx, TLQ_ERR_STATE, "cooling table not set");
  const long long N = o.nsamples;
  const long long Nval = std::max<long long>(o.batch, N / 100);
  const long long Ntr = N - Nval;
  float norm[6];
  for (int q = 0; q < 3; ++q) {
    norm[2 * q] = (float)(0.5 * (o.box[2 * q] + o.box[2 * q + 1]));
    norm[2 * q + 1] = (float)(0.5 * (o.box[2 * q + 1] - o.box[2 * q]));
  }
  cudaStream_t s = ctx->stream;
  float *X = nullptr, *Y = nullptr, *X2 = nullptr, *Y2 = nullptr, *P = nullptr, *m = nullptr, *v = nullptr,
        *grad = nullptr, *loss = nullptr, *Yp = nullptr, *Wt = nullptr, *Wt2 = nullptr;
  long long* perm = nullptr;
  int rc = TLQ_OK;
  auto t0 = std::chrono::steady_clock::now();
  auto cleanup = [&]() {
    cudaFree(X); cudaFree(Y); cudaFree(X2); cudaFree(Y2); cudaFree(m); cudaFree(v); cudaFree(grad);
    cudaFree(Wt); cudaFree(Wt2);
    cudaFree(loss); cudaFree(Yp); cudaFree(perm);
  };
#define TCK(call)                                                                              \
  do {                                                                                         \
    cudaError_t e_ = (call);                                                                   \
    if (e_ != cudaSuccess) {                                                                   \
      cleanup();                                                                               \
      cudaFree(P);                                                                             \
      return sfail(ctx, TLQ_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));     \
    }                                                                                          \
  } while (0)
  TCK(cudaMalloc(&X, 3 * N * sizeof(float)));
  TCK(cudaMalloc(&Y, N * sizeof(float)));
  TCK(cudaMalloc(&X2, 3 * N * sizeof(float)));
  TCK(cudaMalloc(&Y2, N * sizeof(float)));
  TCK(cudaMalloc(&Wt, N * sizeof(float)));
  TCK(cudaMalloc(&Wt2, N * sizeof(float)));
  TCK(cudaMalloc(&perm, N * sizeof(long long)));
  TCK(cudaMalloc(&P, NPARAM * sizeof(float)));
  TCK(cudaMalloc(&m, NPARAM * sizeof(float)));
  TCK(cudaMalloc(&v, NPARAM * sizeof(float)));
  TCK(cudaMalloc(&grad, NPARAM * sizeof(float)));
  TCK(cudaMalloc(&loss, sizeof(float)));
  TCK(cudaMalloc(&Yp, Nval * sizeof(float)));
  // pairs (stratified in tau), shuffled, normalised
  const Params pe = exact_params(ctx, o.sub_frac, o.max_sub);
  TCK(launch_cool_pairs(pe, N, o.seed, o.box, X, Y, Wt, nullptr, s));
  {
    std::vector<long long> hp(N);
    std::iota(hp.begin(), hp.end(), 0LL);
    std::mt19937_64 rng(o.seed * 2654435761ULL + 7);
    std::shuffle(hp.begin(), hp.end(), rng);
    TCK(cudaMemcpyAsync(perm, hp.data(), N * sizeof(long long), cudaMemcpyHostToDevice, s));
    TCK(launch_gather_pairs(X, Y, Wt, perm, N, X2, Y2, Wt2, s));
    TCK(cudaStreamSynchronize(s));
  }
  auto t1 = std::chrono::steady_clock::now();
  TCK(launch_normalise(X2, N, norm, s));
  std::vector<float> hP(NPARAM);
  init_params(hP, o.seed);
  TCK(cudaMemcpyAsync(P, hP.data(), NPARAM * sizeof(float), cudaMemcpyHostToDevice, s));
  TCK(cudaMemsetAsync(m, 0, NPARAM * sizeof(float), s));
  TCK(cudaMemsetAsync(v, 0, NPARAM * sizeof(float), s));
  const long long steps_per_epoch = Ntr / o.batch;
  const long long total = steps_per_epoch * o.epochs;
  const int gblocks = std::max(1, std::min(152 * 2, (o.batch / 16 + 3) / 4));  // 16-sample tiles, 4 warps a block
  float lfirst = 0.f, llast = 0.f;
  long long t = 0;
  for (int ep = 0; ep < o.epochs; ++ep) {
    for (long long b = 0; b < steps_per_epoch; ++b) {
      ++t;
      const float lr = o.lr * (0.05f + 0.95f * 0.5f * (1.0f + std::cos(3.14159265f * (float)(t - 1) / (float)total)));
      TCK(cudaMemsetAsync(grad, 0, NPARAM * sizeof(float), s));
      TCK(cudaMemsetAsync(loss, 0, sizeof(float), s));
      TCK(launch_mlp_grad(P, X2 + 3 * b * o.batch, Y2 + b * o.batch, Wt2 + b * o.batch, o.batch, grad, loss,
                          gblocks, s));
      TCK(launch_adam(P, m, v, grad, NPARAM, lr, 0.9f, 0.999f, 1e-8f, (int)t, s));
      if (t == 1) {
        TCK(cudaMemcpyAsync(&lfirst, loss, sizeof(float), cudaMemcpyDeviceToHost, s));
        TCK(cudaStreamSynchronize(s));
      }
    }
  }
  TCK(cudaMemcpyAsync(&llast, loss, sizeof(float), cudaMemcpyDeviceToHost, s));
  // held-out pairs
  TCK(launch_mlp_infer(P, X2 + 3 * Ntr, (int)Nval, Yp, s));
  std::vector<float> hx(3 * Nval), hy(Nval), hyp(Nval), hw(Nval);
  TCK(cudaMemcpyAsync(hw.data(), Wt2 + Ntr, Nval * sizeof(float), cudaMemcpyDeviceToHost, s));
  TCK(cudaMemcpyAsync(hx.data(), X2 + 3 * Ntr, 3 * Nval * sizeof(float), cudaMemcpyDeviceToHost, s));
  TCK(cudaMemcpyAsync(hy.data(), Y2 + Ntr, Nval * sizeof(float), cudaMemcpyDeviceToHost, s));
  TCK(cudaMemcpyAsync(hyp.data(), Yp, Nval * sizeof(float), cudaMemcpyDeviceToHost, s));
  TCK(cudaStreamSynchronize(s));
  auto t2 = std::chrono::steady_clock::now();
  // held-out pairs that do not complete (the step's network cells): T_new/T
  // as the step forms it (clamped at the table's first temperature)
  double se = 0.0, mx = 0.0;
  std::vector<double> rel;
  rel.reserve(Nval);
  for (long long q = 0; q < Nval; ++q) {
    if (!(hw[q] > 0.0f)) continue;
    const double T = std::pow(10.0, (double)hx[3 * q + 1] * norm[3] + norm[2]);
    const double tau = std::pow(10.0, (double)hx[3 * q + 2] * norm[5] + norm[4]);
    const double d = tau * ((double)hyp[q] - (double)hy[q]);  // error of y = 1 + tau r
    se += d * d;
    // network output r: T_new/T = exp(-(tau + tau^2 r))
    const double pred = std::max(std::exp(-(tau + tau * tau * (double)hyp[q])), ctx->cool_tmin / T);
    rel.push_back(std::fabs(pred - std::exp(-(tau + tau * tau * (double)hy[q]))));  // |dT|/T
    mx = std::max(mx, rel.back());
  }
  if (rel.empty()) rel.push_back(0.0);
  std::sort(rel.begin(), rel.end());
  if (!ctx->mlp_image && cudaMalloc(&ctx->mlp_image, tlq::mlp_image_bytes()) != cudaSuccess) {
    cleanup();
    cudaFree(P);
    return sfail(ctx, TLQ_ERR_NOMEM, "network image");  // (the previous network, if any, stays)
  }
  cudaFree(ctx->mlp_params);
  ctx->mlp_params = P;
  if (tlq::launch_pack_weights(P, ctx->mlp_image, s) != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess) {
    cleanup();
    ctx->mlp_ready = false;
    return sfail(ctx, TLQ_ERR_CUDA, "network image");
  }
  for (int q = 0; q < 6; ++q) {
    ctx->mlp_norm[q] = norm[q];
    ctx->mlp_box[q] = o.box[q];
  }
  ctx->mlp_ready = true;
  invalidate_graphs(ctx);
  if (rep) {
    rep->loss_first = lfirst;
    rep->loss_last = llast;
    rep->val_rmse_y = std::sqrt(se / (double)rel.size());
    rep->val_max_rel_T = mx;
    rep->val_p99_rel_T = rel[(size_t)(0.99 * (double)(rel.size() - 1))];
    rep->val_accept = (double)(std::upper_bound(rel.begin(), rel.end(), 1e-3) - rel.begin()) / (double)rel.size();
    rep->ms_generate = std::chrono::duration<double, std::milli>(t1 - t0).count();
    rep->ms_train = std::chrono::duration<double, std::milli>(t2 - t1).count();
    rep->steps = t;
  }
  cleanup();
#undef TCK
  return rc;
}

int tlq_get_cooling_surrogate(tlq_ctx* ctx, float* params, float* norm6, double* box6) {
  if (!ctx) return TLQ_ERR_ARG;
  if (!ctx->mlp_ready) return sfail(ctx, TLQ_ERR_STATE, "no cooling surrogate");
  if (params) SCK(cudaMemcpy(params, ctx->mlp_params, tlq::mlp::NPARAM * sizeof(float), cudaMemcpyDeviceToHost));
  if (norm6) std::memcpy(norm6, ctx->mlp_norm, 6 * sizeof(float));
  if (box6) std::memcpy(box6, ctx->mlp_box, 6 * sizeof(double));
  return TLQ_OK;
}

int tlq_set_cooling_surrogate(tlq_ctx* ctx, const float* params, const float* norm6, const double* box6) {
  if (!ctx || !params || !norm6 || !box6) return TLQ_ERR_ARG;
  ctx->mlp_ready = false;  // until the parameters and their image are the new network's
  if (!ctx->mlp_params) SCK(cudaMalloc(&ctx->mlp_params, tlq::mlp::NPARAM * sizeof(float)));
  SCK(cudaMemcpy(ctx->mlp_params, params, tlq::mlp::NPARAM * sizeof(float), cudaMemcpyHostToDevice));
  if (!ctx->mlp_image) SCK(cudaMalloc(&ctx->mlp_image, tlq::mlp_image_bytes()));
  SCK(tlq::launch_pack_weights(ctx->mlp_params, ctx->mlp_image, ctx->stream));
  SCK(cudaStreamSynchronize(ctx->stream));
  std::memcpy(ctx->mlp_norm, norm6, 6 * sizeof(float));
  std::memcpy(ctx->mlp_box, box6, 6 * sizeof(double));
  ctx->mlp_ready = true;
  invalidate_graphs(ctx);
  return TLQ_OK;
}

int tlq_mlp_loss_grad(const float* params, const float* X, const float* Y, const float* Wt, int n, float* grad,
                      float* loss) {
  if (!params || !X || !Y || n < 1 || !grad || !loss) return TLQ_ERR_ARG;
  float *dP = nullptr, *dX = nullptr, *dY = nullptr, *dW = nullptr, *dg = nullptr, *dl = nullptr;
  cudaError_t e = cudaMalloc(&dP, tlq::mlp::NPARAM * sizeof(float));
  if (e == cudaSuccess && Wt) e = cudaMalloc(&dW, (size_t)n * sizeof(float));
  if (e == cudaSuccess && Wt) e = cudaMemcpy(dW, Wt, (size_t)n * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMalloc(&dX, 3 * (size_t)n * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&dY, (size_t)n * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&dg, tlq::mlp::NPARAM * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&dl, sizeof(float));
  if (e == cudaSuccess) e = cudaMemcpy(dP, params, tlq::mlp::NPARAM * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dX, X, 3 * (size_t)n * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dY, Y, (size_t)n * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(dg, 0, tlq::mlp::NPARAM * sizeof(float));
  if (e == cudaSuccess) e = cudaMemset(dl, 0, sizeof(float));
  if (e == cudaSuccess)
    e = launch_mlp_grad(dP, dX, dY, dW, n, dg, dl, std::max(1, std::min(152 * 2, (n / 16 + 3) / 4)), 0);
  if (e == cudaSuccess) e = cudaMemcpy(grad, dg, tlq::mlp::NPARAM * sizeof(float), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(loss, dl, sizeof(float), cudaMemcpyDeviceToHost);
  cudaFree(dP); cudaFree(dX); cudaFree(dY); cudaFree(dW); cudaFree(dg); cudaFree(dl);
  return e == cudaSuccess ? TLQ_OK : TLQ_ERR_CUDA;
}

int tlq_mlp_infer(const float* params, const float* X, int n, float* Yout) {
  if (!params || !X || n < 1 || !Yout) return TLQ_ERR_ARG;
  float *dP = nullptr, *dX = nullptr, *dY = nullptr;
  cudaError_t e = cudaMalloc(&dP, tlq::mlp::NPARAM * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&dX, 3 * (size_t)n * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&dY, (size_t)n * sizeof(float));
  if (e == cudaSuccess) e = cudaMemcpy(dP, params, tlq::mlp::NPARAM * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dX, X, 3 * (size_t)n * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = launch_mlp_infer(dP, dX, n, dY, 0);
  if (e == cudaSuccess) e = cudaMemcpy(Yout, dY, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost);
  cudaFree(dP); cudaFree(dX); cudaFree(dY);
  return e == cudaSuccess ? TLQ_OK : TLQ_ERR_CUDA;
}

}  // extern "C"
