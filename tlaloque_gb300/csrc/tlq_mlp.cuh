// tlq_mlp.cuh -- the learned cooling surrogate: a 3-64-64-64-1 SiLU MLP run
// on the tensor cores with BF16 operands and FP32 accumulation.
//
// One warp evaluates 32 samples (two m16 row tiles) with mma.sync
// m16n8k16.bf16.  The FP32 accumulator fragment of a layer is, element for
// element, the A-operand fragment of the next layer (the thread that holds
// output columns 16kt..16kt+15 of a row holds exactly the operand slice of
// k-tile kt), so activations never leave registers in the forward pass.
// Weights live in shared memory as BF16, rows padded to 72 (conflict-free
// 32-bit operand loads).  The 3 -> 64 input layer and the 64 -> 1 output
// layer are FP32 dot products (FP32 weights, inputs and activations): they
// are 4 % of the work, and BF16 inputs (2^-9 of the normalised log features,
// i.e. 1-2 % in T and tau) or a BF16 output would cost the most accuracy.
#pragma once

#include <cuda_bf16.h>

#include <cstdint>

namespace tlq {
namespace mlp {

constexpr int IN = 3, HID = 64;
constexpr int LD = HID + 8;  // padded row length (bf16) of the 64-wide weights
// FP32 master parameters, packed: W1[64][3] b1[64] W2[64][64] b2[64] W3[64][64] b3[64] W4[64] b4
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + HID * IN, OFF_W2 = OFF_B1 + HID, OFF_B2 = OFF_W2 + HID * HID,
              OFF_W3 = OFF_B2 + HID, OFF_B3 = OFF_W3 + HID * HID, OFF_W4 = OFF_B3 + HID, OFF_B4 = OFF_W4 + HID,
              NPARAM = OFF_B4 + 1;  // 8641

// Weights of one network in shared memory (BF16, padded) plus FP32 biases.
struct alignas(16) SmemWeights {
  float w1[HID][4];             // input layer, FP32 (out x in, in padded 3 -> 4; rows read as float4)
  __nv_bfloat16 w2[HID][LD];
  __nv_bfloat16 w3[HID][LD];
  float w4[HID];                // output layer, FP32
  float b1[HID], b2[HID], b3[HID], b4;
};
// Transposed copies for the backward pass (dH = dZ W).
struct SmemWeightsT {
  __nv_bfloat16 w2t[HID][LD];
  __nv_bfloat16 w3t[HID][LD];
};

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);  // .x = lo (low 16 bits)
  return *reinterpret_cast<const uint32_t*>(&v);
}
__device__ __forceinline__ float bf16r(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

__device__ __forceinline__ void mma_bf16(float* d, const uint32_t* a, uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
      "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ float sigmoid_f(float z) { return 1.0f / (1.0f + __expf(-z)); }
__device__ __forceinline__ float silu_f(float z) { return z * sigmoid_f(z); }
__device__ __forceinline__ float dsilu_f(float z) {
  const float s = sigmoid_f(z);
  return s * (1.0f + z * (1.0f - s));
}

// Load the FP32 master parameters into the BF16 shared layout (all threads).
__device__ inline void load_weights(const float* __restrict__ P, SmemWeights& W, SmemWeightsT* WT) {
  for (int q = threadIdx.x; q < HID * 4; q += blockDim.x) {
    const int n = q / 4, k = q % 4;
    W.w1[n][k] = k < IN ? P[OFF_W1 + n * IN + k] : 0.0f;
  }
  for (int q = threadIdx.x; q < HID * LD; q += blockDim.x) {
    const int n = q / LD, k = q % LD;
    const bool in = k < HID;
    W.w2[n][k] = __float2bfloat16_rn(in ? P[OFF_W2 + n * HID + k] : 0.0f);
    W.w3[n][k] = __float2bfloat16_rn(in ? P[OFF_W3 + n * HID + k] : 0.0f);
    if (WT) {
      WT->w2t[n][k] = __float2bfloat16_rn(in ? P[OFF_W2 + k * HID + n] : 0.0f);
      WT->w3t[n][k] = __float2bfloat16_rn(in ? P[OFF_W3 + k * HID + n] : 0.0f);
    }
  }
  for (int q = threadIdx.x; q < HID; q += blockDim.x) {
    W.w4[q] = P[OFF_W4 + q];
    W.b1[q] = P[OFF_B1 + q];
    W.b2[q] = P[OFF_B2 + q];
    W.b3[q] = P[OFF_B3 + q];
  }
  if (threadIdx.x == 0) W.b4 = P[OFF_B4];
}

// A block's copy of a network image that pack_weights (tlq_mlp.cu) formed
// once in device memory with load_weights: 16-byte loads, all of a thread's
// issued before the first store, instead of load_weights' scalar gathers
// and conversions in every block.  Same bytes, so the same results.
template <int NT>
__device__ __forceinline__ void copy_weights(const SmemWeights* __restrict__ img, SmemWeights& W) {
  constexpr int NV = (int)(sizeof(SmemWeights) / 16), R = (NV + NT - 1) / NT;
  const uint4* __restrict__ src = reinterpret_cast<const uint4*>(img);
  uint4* dst = reinterpret_cast<uint4*>(&W);
  uint4 v[R];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int q = (int)threadIdx.x + r * NT;
    if (q < NV) v[r] = __ldg(src + q);
  }
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int q = (int)threadIdx.x + r * NT;
    if (q < NV) dst[q] = v[r];
  }
}

// Input layer in FP32 for one m16 tile, straight into the accumulator
// layout: acc[j] = (rows g, g+8) x (columns 8j+2tig, 8j+2tig+1).
__device__ __forceinline__ void input_layer(float acc[8][4], const SmemWeights& W, const float* xg, const float* xg8,
                                            int tig) {
#pragma unroll
  for (int j = 0; j < 8; ++j) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int c = 8 * j + 2 * tig + h;
      const float4 w = *reinterpret_cast<const float4*>(W.w1[c]);
      acc[j][h] = W.b1[c] + w.x * xg[0] + w.y * xg[1] + w.z * xg[2];
      acc[j][2 + h] = W.b1[c] + w.x * xg8[0] + w.y * xg8[1] + w.z * xg8[2];
    }
  }
}

// One dense layer with K = 16*KT inputs and 64 outputs for one m16 tile:
// acc[j][0..3] = bias + A x W^T (n-tile j = output columns 8j..8j+7).
template <int KT, int LDW>
__device__ __forceinline__ void dense64(float acc[8][4], const uint32_t (*a)[4], const __nv_bfloat16 (*w)[LDW],
                                        const float* bias, int g, int tig) {
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const float b0 = bias ? bias[8 * j + 2 * tig] : 0.0f, b1v = bias ? bias[8 * j + 2 * tig + 1] : 0.0f;
    acc[j][0] = b0; acc[j][1] = b1v; acc[j][2] = b0; acc[j][3] = b1v;
#pragma unroll
    for (int kt = 0; kt < KT; ++kt) {
      const uint32_t bb0 = *reinterpret_cast<const uint32_t*>(&w[8 * j + g][16 * kt + 2 * tig]);
      const uint32_t bb1 = *reinterpret_cast<const uint32_t*>(&w[8 * j + g][16 * kt + 2 * tig + 8]);
      mma_bf16(acc[j], a[kt], bb0, bb1);
    }
  }
}

// Accumulator fragments (pre-activation z) -> SiLU -> next layer's operand
// fragments (BF16).
__device__ __forceinline__ void act_to_frag(uint32_t a[4][4], const float z[8][4]) {
#pragma unroll
  for (int kt = 0; kt < 4; ++kt) {
    const float* c0 = z[2 * kt];
    const float* c1 = z[2 * kt + 1];
    a[kt][0] = pack_bf16(silu_f(c0[0]), silu_f(c0[1]));
    a[kt][1] = pack_bf16(silu_f(c0[2]), silu_f(c0[3]));
    a[kt][2] = pack_bf16(silu_f(c1[0]), silu_f(c1[1]));
    a[kt][3] = pack_bf16(silu_f(c1[2]), silu_f(c1[3]));
  }
}

// Forward pass of one m16 tile; returns the outputs of rows g and g+8 in
// y[0], y[1] (in all four lanes of the group g).  Optionally keeps the
// pre-activations of the three hidden layers (training).
__device__ __forceinline__ void forward_tile(const SmemWeights& W, const float* xg, const float* xg8, int g, int tig,
                                             float* y, float (*z1)[4] = nullptr, float (*z2)[4] = nullptr,
                                             float (*z3)[4] = nullptr) {
  float acc[8][4];
  input_layer(acc, W, xg, xg8, tig);
  if (z1) {
#pragma unroll
    for (int j = 0; j < 8; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) z1[j][q] = acc[j][q];
  }
  uint32_t a[4][4];
  act_to_frag(a, acc);
  dense64<4, LD>(acc, a, W.w2, W.b2, g, tig);
  if (z2) {
#pragma unroll
    for (int j = 0; j < 8; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) z2[j][q] = acc[j][q];
  }
  act_to_frag(a, acc);
  dense64<4, LD>(acc, a, W.w3, W.b3, g, tig);
  if (z3) {
#pragma unroll
    for (int j = 0; j < 8; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) z3[j][q] = acc[j][q];
  }
  // output layer in FP32: this lane's 16 columns, then the sum over tig
  float s0 = 0.0f, s1 = 0.0f;
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const int c = 8 * j + 2 * tig;
    s0 += W.w4[c] * silu_f(acc[j][0]) + W.w4[c + 1] * silu_f(acc[j][1]);
    s1 += W.w4[c] * silu_f(acc[j][2]) + W.w4[c + 1] * silu_f(acc[j][3]);
  }
  s0 += __shfl_xor_sync(0xffffffffu, s0, 1);
  s1 += __shfl_xor_sync(0xffffffffu, s1, 1);
  s0 += __shfl_xor_sync(0xffffffffu, s0, 2);
  s1 += __shfl_xor_sync(0xffffffffu, s1, 2);
  y[0] = W.b4 + s0;  // row g
  y[1] = W.b4 + s1;  // row g + 8
}

}  // namespace mlp
}  // namespace tlq
