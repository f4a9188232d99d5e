// tlq_mlp.cu -- training and inference kernels of the cooling surrogate, and
// the generator of its training pairs (the exact, finely sub-cycled form of
// the reference's cooling step, source/cooling.f90:64-112, in FP64).
//
// Numerics (mirrored by the CPU oracle oracle/mlp_oracle.py): the weights of
// the hidden layers 2 and 3 and every activation fed to a tensor-core
// product are rounded to BF16; products accumulate in FP32; the input and
// output layers, biases, pre-activations, SiLU derivatives, the loss
// gradient, the layer-1 and layer-4 weight gradients are FP32.
#include "tlq_internal.h"
#include "tlq_mlp.cuh"
#include "tlq_umma.cuh"

namespace tlq {
namespace mlp {

constexpr int TW = 4;        // warps per training block
constexpr int TT = TW * 32;  // threads per training block
constexpr int TS = 16;       // samples per warp tile
constexpr int LDS = TS + 8;  // padded row length of the transposed staging tiles

struct TrainSmem {
  SmemWeights W;
  SmemWeightsT WT;
  __nv_bfloat16 stA[TW][HID][LDS];  // dZ^T of the tile (features x samples)
  __nv_bfloat16 stB[TW][HID][LDS];  // H^T of the tile
  float g[NPARAM];                  // this block's gradient
  float loss;
};

__device__ __forceinline__ void frag_plain(uint32_t a[4][4], const float d[8][4]) {
#pragma unroll
  for (int kt = 0; kt < 4; ++kt) {
    a[kt][0] = pack_bf16(d[2 * kt][0], d[2 * kt][1]);
    a[kt][1] = pack_bf16(d[2 * kt][2], d[2 * kt][3]);
    a[kt][2] = pack_bf16(d[2 * kt + 1][0], d[2 * kt + 1][1]);
    a[kt][3] = pack_bf16(d[2 * kt + 1][2], d[2 * kt + 1][3]);
  }
}

// Sum over the 8 lanes that share tig (rows g = 0..7 of a fragment).
__device__ __forceinline__ float sum_over_g(float v) {
  v += __shfl_xor_sync(0xffffffffu, v, 4);
  v += __shfl_xor_sync(0xffffffffu, v, 8);
  v += __shfl_xor_sync(0xffffffffu, v, 16);
  return v;
}

// dW_layer (64 x 64, out x in) += dZ^T H over the warp's 16 samples, from the
// transposed BF16 staging tiles, into the block gradient (shared atomics).
__device__ __forceinline__ void weight_grad64(float* gW, const __nv_bfloat16 (*dzT)[LDS],
                                              const __nv_bfloat16 (*hT)[LDS], int g, int tig) {
#pragma unroll
  for (int mt = 0; mt < 4; ++mt) {  // output-feature tile (rows of dW)
    uint32_t a[4];
    a[0] = *reinterpret_cast<const uint32_t*>(&dzT[16 * mt + g][2 * tig]);
    a[1] = *reinterpret_cast<const uint32_t*>(&dzT[16 * mt + g + 8][2 * tig]);
    a[2] = *reinterpret_cast<const uint32_t*>(&dzT[16 * mt + g][2 * tig + 8]);
    a[3] = *reinterpret_cast<const uint32_t*>(&dzT[16 * mt + g + 8][2 * tig + 8]);
#pragma unroll
    for (int j = 0; j < 8; ++j) {  // input-feature tile (columns of dW)
      float acc[4] = {0.f, 0.f, 0.f, 0.f};
      const uint32_t b0 = *reinterpret_cast<const uint32_t*>(&hT[8 * j + g][2 * tig]);
      const uint32_t b1 = *reinterpret_cast<const uint32_t*>(&hT[8 * j + g][2 * tig + 8]);
      mma_bf16(acc, a, b0, b1);
      const int r0 = 16 * mt + g, c0 = 8 * j + 2 * tig;
      atomicAdd(&gW[r0 * HID + c0], acc[0]);
      atomicAdd(&gW[r0 * HID + c0 + 1], acc[1]);
      atomicAdd(&gW[(r0 + 8) * HID + c0], acc[2]);
      atomicAdd(&gW[(r0 + 8) * HID + c0 + 1], acc[3]);
    }
  }
}

// Stage a C-layout fragment set (rows = samples g, g+8; 64 features) as the
// transposed BF16 tile [feature][sample].
__device__ __forceinline__ void stage_T(__nv_bfloat16 (*dst)[LDS], const float v[8][4], int g, int tig) {
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const int c = 8 * j + 2 * tig;
    dst[c][g] = __float2bfloat16_rn(v[j][0]);
    dst[c + 1][g] = __float2bfloat16_rn(v[j][1]);
    dst[c][g + 8] = __float2bfloat16_rn(v[j][2]);
    dst[c + 1][g + 8] = __float2bfloat16_rn(v[j][3]);
  }
}

// One pass over a minibatch: loss sum_i |w_i| e_i^2 / nb and its gradient
// w.r.t. the FP32 parameters P, on features X (3 per sample, normalised),
// targets Y and weights Wt (all 1 when null), e_i = y_i - t_i, or
// min(y_i - t_i, 0) where w_i < 0 (a one-sided target: y_i >= t_i).  grad and
// loss are accumulated with global atomics.
__global__ void __launch_bounds__(TT) k_mlp_grad(const float* __restrict__ P, const float* __restrict__ X,
                                                 const float* __restrict__ Y, const float* __restrict__ Wt, int nb,
                                                 float* grad, float* loss) {
  extern __shared__ __align__(16) unsigned char sm_[];
  TrainSmem& s = *reinterpret_cast<TrainSmem*>(sm_);
  load_weights(P, s.W, &s.WT);
  for (int q = threadIdx.x; q < NPARAM; q += TT) s.g[q] = 0.0f;
  if (threadIdx.x == 0) s.loss = 0.0f;
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, tig = lane & 3;
  const float inv_nb = 1.0f / (float)nb;
  const int ntiles = (nb + TS - 1) / TS;
  for (int tile = blockIdx.x * TW + warp; tile < ntiles; tile += gridDim.x * TW) {
    const int r0 = tile * TS + g, r1 = r0 + 8;
    const bool v0 = r0 < nb, v1 = r1 < nb;
    float xg[3] = {0.f, 0.f, 0.f}, xg8[3] = {0.f, 0.f, 0.f};
    if (v0) for (int f = 0; f < 3; ++f) xg[f] = X[3 * r0 + f];
    if (v1) for (int f = 0; f < 3; ++f) xg8[f] = X[3 * r1 + f];
    float z1[8][4], z2[8][4], z3[8][4], y[2];
    forward_tile(s.W, xg, xg8, g, tig, y, z1, z2, z3);
    // d loss / d y = 2 w (y - t) / nb (rows outside the batch contribute 0)
    float dy0 = 0.f, dy1 = 0.f;
    if (tig == 0) {
      float w0 = v0 ? (Wt ? Wt[r0] : 1.0f) : 0.0f, w1 = v1 ? (Wt ? Wt[r1] : 1.0f) : 0.0f;
      float e0 = v0 ? y[0] - Y[r0] : 0.0f, e1 = v1 ? y[1] - Y[r1] : 0.0f;
      if (w0 < 0.0f) { w0 = -w0; e0 = fminf(e0, 0.0f); }
      if (w1 < 0.0f) { w1 = -w1; e1 = fminf(e1, 0.0f); }
      dy0 = 2.0f * w0 * e0 * inv_nb;
      dy1 = 2.0f * w1 * e1 * inv_nb;
      atomicAdd(&s.loss, (w0 * e0 * e0 + w1 * e1 * e1) * inv_nb);
    }
    dy0 = __shfl_sync(0xffffffffu, dy0, lane & ~3);
    dy1 = __shfl_sync(0xffffffffu, dy1, lane & ~3);
    // layer 4: dW4 = dy H3, db4 = sum dy, dZ3 = dy W4 * silu'(z3)
    float d[8][4];
    float db4p = (tig == 0) ? dy0 + dy1 : 0.0f;
    db4p = sum_over_g(db4p);
    if (lane == 0) atomicAdd(&s.g[OFF_B4], db4p);
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int c = 8 * j + 2 * tig;
      const float w0 = s.W.w4[c], w1v = s.W.w4[c + 1];
      const float h00 = silu_f(z3[j][0]), h01 = silu_f(z3[j][1]);
      const float h10 = silu_f(z3[j][2]), h11 = silu_f(z3[j][3]);
      float gw0 = sum_over_g(dy0 * h00 + dy1 * h10);
      float gw1 = sum_over_g(dy0 * h01 + dy1 * h11);
      if (g == 0) {
        atomicAdd(&s.g[OFF_W4 + c], gw0);
        atomicAdd(&s.g[OFF_W4 + c + 1], gw1);
      }
      d[j][0] = dy0 * w0 * dsilu_f(z3[j][0]);
      d[j][1] = dy0 * w1v * dsilu_f(z3[j][1]);
      d[j][2] = dy1 * w0 * dsilu_f(z3[j][2]);
      d[j][3] = dy1 * w1v * dsilu_f(z3[j][3]);
    }
    // layers 3 and 2: db = sum dZ; dW = dZ^T H (tensor cores); dH = dZ W (tensor cores)
    const int offW[2] = {OFF_W3, OFF_W2}, offB[2] = {OFF_B3, OFF_B2};
#pragma unroll
    for (int L = 0; L < 2; ++L) {
      float (*zin)[4] = (L == 0) ? z2 : z1;  // pre-activation feeding this layer
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int c = 8 * j + 2 * tig;
        const float s0 = sum_over_g(d[j][0] + d[j][2]);
        const float s1 = sum_over_g(d[j][1] + d[j][3]);
        if (g == 0) {
          atomicAdd(&s.g[offB[L] + c], s0);
          atomicAdd(&s.g[offB[L] + c + 1], s1);
        }
      }
      float h[8][4];
#pragma unroll
      for (int j = 0; j < 8; ++j)
#pragma unroll
        for (int q = 0; q < 4; ++q) h[j][q] = silu_f(zin[j][q]);
      __syncwarp();
      stage_T(s.stA[warp], d, g, tig);
      stage_T(s.stB[warp], h, g, tig);
      __syncwarp();
      weight_grad64(&s.g[offW[L]], s.stA[warp], s.stB[warp], g, tig);
      __syncwarp();
      uint32_t a[4][4];
      frag_plain(a, d);
      float dh[8][4];
      if (L == 0)
        dense64<4, LD>(dh, a, s.WT.w3t, nullptr, g, tig);
      else
        dense64<4, LD>(dh, a, s.WT.w2t, nullptr, g, tig);
#pragma unroll
      for (int j = 0; j < 8; ++j)
#pragma unroll
        for (int q = 0; q < 4; ++q) d[j][q] = dh[j][q] * dsilu_f(zin[j][q]);
    }
    // layer 1: db1 = sum dZ1, dW1 = dZ1^T X (K = 3, FP32)
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int c = 8 * j + 2 * tig;
      const float s0 = sum_over_g(d[j][0] + d[j][2]);
      const float s1 = sum_over_g(d[j][1] + d[j][3]);
      if (g == 0) {
        atomicAdd(&s.g[OFF_B1 + c], s0);
        atomicAdd(&s.g[OFF_B1 + c + 1], s1);
      }
#pragma unroll
      for (int f = 0; f < 3; ++f) {
        const float w0 = sum_over_g(d[j][0] * xg[f] + d[j][2] * xg8[f]);
        const float w1v = sum_over_g(d[j][1] * xg[f] + d[j][3] * xg8[f]);
        if (g == 0) {
          atomicAdd(&s.g[OFF_W1 + c * IN + f], w0);
          atomicAdd(&s.g[OFF_W1 + (c + 1) * IN + f], w1v);
        }
      }
    }
  }
  __syncthreads();
  for (int q = threadIdx.x; q < NPARAM; q += TT) atomicAdd(&grad[q], s.g[q]);
  if (threadIdx.x == 0) atomicAdd(loss, s.loss);
}

// Adam on the FP32 master parameters.
__global__ void k_adam(float* P, float* m, float* v, const float* grad, int n, float lr, float b1, float b2,
                       float eps, float c1, float c2) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const float gq = grad[q];
  const float mq = b1 * m[q] + (1.0f - b1) * gq;
  const float vq = b2 * v[q] + (1.0f - b2) * gq * gq;
  m[q] = mq;
  v[q] = vq;
  P[q] -= lr * (mq / c1) / (sqrtf(vq / c2) + eps);
}

// Batch inference (features normalised, 3 per sample) -> y.
__global__ void __launch_bounds__(TT) k_mlp_infer(const float* __restrict__ P, const float* __restrict__ X, int n,
                                                  float* __restrict__ Yout) {
  __shared__ SmemWeights W;
  load_weights(P, W, nullptr);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, tig = lane & 3;
  const int ntiles = (n + TS - 1) / TS;
  for (int tile = blockIdx.x * TW + warp; tile < ntiles; tile += gridDim.x * TW) {
    const int r0 = tile * TS + g, r1 = r0 + 8;
    float xg[3] = {0.f, 0.f, 0.f}, xg8[3] = {0.f, 0.f, 0.f};
    if (r0 < n) for (int f = 0; f < 3; ++f) xg[f] = X[3 * r0 + f];
    if (r1 < n) for (int f = 0; f < 3; ++f) xg8[f] = X[3 * r1 + f];
    float y[2];
    forward_tile(W, xg, xg8, g, tig, y);
    if (tig == 0) {
      if (r0 < n) Yout[r0] = y[0];
      if (r1 < n) Yout[r1] = y[1];
    }
  }
}

// Batch inference on the tcgen05 path of the step's network pass
// (tlq_umma.cuh): 128 samples per tile, one per thread.  A tile whose MMA
// wait ran out writes NaN (the caller sees it), and the block stops.
__global__ void __launch_bounds__(umma::ROWS) k_mlp_infer_umma(const float* __restrict__ P,
                                                               const float* __restrict__ X, int n,
                                                               float* __restrict__ Yout) {
  __shared__ umma::Smem S;
  const int ntiles = (n + umma::ROWS - 1) / umma::ROWS;
  if ((int)blockIdx.x >= ntiles) return;
  umma::load_weights_fp32(P, S);
  umma::setup(S);
  uint32_t phase = 0;
  bool tc = true;
  for (int tile = blockIdx.x; tile < ntiles && tc; tile += gridDim.x) {
    const int r = tile * umma::ROWS + (int)threadIdx.x;
    float x[3] = {0.f, 0.f, 0.f};
    if (r < n)
      for (int f = 0; f < 3; ++f) x[f] = X[3 * r + f];
    float y = 0.f;
    tc = umma::forward(S, x, y, phase);
    if (r < n) Yout[r] = tc ? y : NAN;
  }
  if (!tc) umma::drain(S, phase);
  umma::teardown(S);
}

// ---------------------------------------------------------------------------
// Training pairs from the exact integrator.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint64_t mix64(uint64_t x) {  // splitmix64 finaliser
  x += 0x9e3779b97f4a7c15ULL;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ULL;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebULL;
  return x ^ (x >> 31);
}
__device__ __forceinline__ double uniform01(uint64_t seed, uint64_t i, int stream) {
  return (double)(mix64(seed ^ mix64(i * 4 + stream)) >> 11) * (1.0 / 9007199254740992.0);
}

// Sample i of N: log10 n and log10 T uniform in the box, log10 tau (the
// step's cooling number Lambda(T) n^2 dt / E_th) stratified in i so that the
// 32 samples of a warp need similar numbers of sub-steps; dt follows from
// tau.  The pair is (features, r) with r = (y - 1)/tau, y = ln(T/T_new)/tau,
// T_new from the exact integrator's closed form (params' cooling
// COOL_EXACT, FP64) or from the finely sub-cycled FP64 integrator (cool_cell
// with the params' sub-step settings).  ln(T/T_new) = tau + tau^2 r is exact to first
// order whatever r is (y -> 1 as tau -> 0; r -> -(s-1)/2, s the local slope
// of the table), and r is O(1) everywhere; below tau ~ 1e-5 r is lost to
// FP64 round-off (ln(T/T_new) - tau ~ 1e-16 against tau^2), so those pairs
// are weighted (tau/1e-5)^2 -- their tau^2 r is negligible in the step.
// The sub-cycled exponential step is first order in its sub-step, so it is
// run with sub-steps of frac and frac/2 and extrapolated (Richardson):
// ln T_new = 2 ln T_(frac/2) - ln T_(frac), second order -- which still
// leaves it ~1e-5 of T above the exact solution on average (up to 3e-4)
// where cooling runs away (tau ~ 0.1-1: the cooling coefficient grows by
// decades within the step), a one-sided error a network trained on it
// inherits; hence the closed form by default.  A pair whose
// cooling reaches the table's first temperature within the step (cooling
// stops there, cooling.f90:71) is "completed": its target is the y that
// lands exactly on that temperature, with weight 0 (the step hands such
// cells to the integrator, whose last sub-step decides where below that
// temperature they end), so the network need not follow the kink at
// completion.  Other pairs have weight 1.
__global__ void k_cool_pairs(Params p, long long N, uint64_t seed, double lnlo, double lnhi, double ltlo,
                             double lthi, double lclo, double lchi, float* __restrict__ X, float* __restrict__ Y,
                             float* __restrict__ Wt, double* __restrict__ raw) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= N) return;
  const double ln = lnlo + (lnhi - lnlo) * uniform01(seed, i, 0);
  const double lt = ltlo + (lthi - ltlo) * uniform01(seed, i, 1);
  const double lc = lclo + (lchi - lclo) * (((double)i + uniform01(seed, i, 2)) / (double)N);
  const double n = pow(10.0, ln), T = pow(10.0, lt), tau = pow(10.0, lc);
  // state with density n mu0 AMU and temperature T at rest
  double w[5];
  w[0] = n * p.mu0 * AMU;
  w[1] = w[2] = w[3] = 0.0;
  w[4] = w[0] * KB * T / (p.mu0 * AMU);
  const double eth = w[4] / (p.gamma - 1.0);
  const double lam = cool_coef(p.cool, T);
  const double ce = lam * (n * n) / eth;
  const double dt = tau / ce;
  const double Tmin = p.cool.T[0];
  double Tn;
  bool completed;
  if (p.cooling == COOL_EXACT) {
    Tn = cool_exact_T(p.cool, T, lam, tau);
    completed = !(Tn > Tmin);
  } else {
    const double p0 = w[4];
    double u4 = eth;
    cool_cell(p, w, u4, dt);
    const double T1 = w[4] * p.mu0 * AMU / (w[0] * KB);
    Params ph = p;
    ph.cool_sub_frac = 0.5 * p.cool_sub_frac;
    w[4] = p0;
    u4 = eth;
    cool_cell(ph, w, u4, dt);
    const double T2 = w[4] * p.mu0 * AMU / (w[0] * KB);
    Tn = exp(2.0 * log(T2) - log(T1));
    completed = T2 < Tmin || Tn < Tmin;
  }
  if (completed) Tn = Tmin;
  X[3 * i + 0] = (float)ln;
  X[3 * i + 1] = (float)lt;
  X[3 * i + 2] = (float)lc;
  // target r = (y - 1) / tau with y = ln(T / T_new) / tau
  const double r = (-log(Tn / T) - tau) / (tau * tau);
  Y[i] = completed ? 0.0f : (float)r;
  if (Wt) Wt[i] = completed ? 0.0f : (float)fmin(1.0, (tau / 1e-5) * (tau / 1e-5));
  if (raw) {
    raw[4 * i + 0] = n;
    raw[4 * i + 1] = T;
    raw[4 * i + 2] = Tn;
    raw[4 * i + 3] = dt;
  }
}

// Gather a permutation of the pairs (shuffles the stratified order).
__global__ void k_gather_pairs(const float* __restrict__ X, const float* __restrict__ Y, const float* __restrict__ Wt,
                               const long long* perm, long long N, float* __restrict__ X2, float* __restrict__ Y2,
                               float* __restrict__ Wt2) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= N) return;
  const long long j = perm[i];
  X2[3 * i + 0] = X[3 * j + 0];
  X2[3 * i + 1] = X[3 * j + 1];
  X2[3 * i + 2] = X[3 * j + 2];
  Y2[i] = Y[j];
  Wt2[i] = Wt[j];
}

// Normalise raw features (log10 n, log10 T, log10 tau) to [-1, 1] over the box.
__global__ void k_normalise(float* X, long long N, float c0, float h0, float c1, float h1, float c2, float h2) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= N) return;
  X[3 * i + 0] = (X[3 * i + 0] - c0) / h0;
  X[3 * i + 1] = (X[3 * i + 1] - c1) / h1;
  X[3 * i + 2] = (X[3 * i + 2] - c2) / h2;
}

}  // namespace mlp

cudaError_t launch_cool_pairs(const Params& p, long long N, unsigned long long seed, const double box[6], float* X,
                              float* Y, float* Wt, double* raw, cudaStream_t s) {
  const int bt = 128;
  mlp::k_cool_pairs<<<(unsigned)((N + bt - 1) / bt), bt, 0, s>>>(p, N, seed, box[0], box[1], box[2], box[3], box[4],
                                                                  box[5], X, Y, Wt, raw);
  return cudaGetLastError();
}

cudaError_t launch_gather_pairs(const float* X, const float* Y, const float* Wt, const long long* perm, long long N,
                                float* X2, float* Y2, float* Wt2, cudaStream_t s) {
  mlp::k_gather_pairs<<<(unsigned)((N + 255) / 256), 256, 0, s>>>(X, Y, Wt, perm, N, X2, Y2, Wt2);
  return cudaGetLastError();
}

cudaError_t launch_normalise(float* X, long long N, const float norm[6], cudaStream_t s) {
  mlp::k_normalise<<<(unsigned)((N + 255) / 256), 256, 0, s>>>(X, N, norm[0], norm[1], norm[2], norm[3], norm[4],
                                                                norm[5]);
  return cudaGetLastError();
}

size_t mlp_train_smem() { return sizeof(mlp::TrainSmem); }

cudaError_t launch_mlp_grad(const float* P, const float* X, const float* Y, const float* Wt, int nb, float* grad,
                            float* loss, int nblocks, cudaStream_t s) {
  // (set on every call: the attribute belongs to the current device)
  const cudaError_t e = cudaFuncSetAttribute(mlp::k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)sizeof(mlp::TrainSmem));
  if (e != cudaSuccess) return e;
  mlp::k_mlp_grad<<<nblocks, mlp::TT, sizeof(mlp::TrainSmem), s>>>(P, X, Y, Wt, nb, grad, loss);
  return cudaGetLastError();
}

cudaError_t launch_adam(float* P, float* m, float* v, const float* grad, int n, float lr, float b1, float b2,
                        float eps, int t, cudaStream_t s) {
  const float c1 = 1.0f - powf(b1, (float)t), c2 = 1.0f - powf(b2, (float)t);
  mlp::k_adam<<<(n + 255) / 256, 256, 0, s>>>(P, m, v, grad, n, lr, b1, b2, eps, c1, c2);
  return cudaGetLastError();
}

namespace {
__global__ void k_pack_weights(const float* __restrict__ P, mlp::SmemWeights* img) { mlp::load_weights(P, *img, nullptr); }
}  // namespace

size_t mlp_image_bytes() { return sizeof(mlp::SmemWeights); }

cudaError_t launch_pack_weights(const float* P, void* img, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(img, 0, sizeof(mlp::SmemWeights), s);  // (struct padding too)
  if (e != cudaSuccess) return e;
  k_pack_weights<<<1, 256, 0, s>>>(P, static_cast<mlp::SmemWeights*>(img));
  return cudaGetLastError();
}

cudaError_t launch_mlp_infer(const float* P, const float* X, int n, float* Y, cudaStream_t s) {
  // the step's forward pass (tcgen05, TMEM accumulators)
  const int tiles = (n + umma::ROWS - 1) / umma::ROWS;
  const int blocks = std::max(1, std::min(tiles, 152 * 3));
  mlp::k_mlp_infer_umma<<<blocks, umma::ROWS, 0, s>>>(P, X, n, Y);
  return cudaGetLastError();
}

// The mma.sync forward pass (the training kernels' own), for comparison.
cudaError_t launch_mlp_infer_sync(const float* P, const float* X, int n, float* Y, cudaStream_t s) {
  const int tiles = (n + mlp::TS - 1) / mlp::TS;
  const int blocks = std::max(1, std::min((tiles + mlp::TW - 1) / mlp::TW, 152 * 8));
  mlp::k_mlp_infer<<<blocks, mlp::TT, 0, s>>>(P, X, n, Y);
  return cudaGetLastError();
}

}  // namespace tlq
