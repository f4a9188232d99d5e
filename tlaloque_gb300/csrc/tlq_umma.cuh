// tlq_umma.cuh -- the cooling surrogate's forward pass on Blackwell's
// tensor cores (tcgen05): BF16 operands in shared memory, FP32 accumulators
// in tensor memory (TMEM).
//
// One block of 128 threads evaluates 128 cells, one thread per cell (row):
//   layer 1 (3 -> 64, FP32 on the CUDA cores) -> SiLU -> BF16 activations
//     written to shared memory in the MMA's operand layout;
//   layers 2 and 3 (64 -> 64): one elected thread issues four
//     tcgen05.mma.cta_group::1.kind::f16 (M 128, N 64, K 16 each) into 64
//     TMEM columns and commits them to an mbarrier; every thread then reads
//     its own row back (tcgen05.ld.32x32b: warp w reaches TMEM lanes
//     32w..32w+31, i.e. rows 32w..32w+31), adds the bias and applies SiLU;
//   layer 4 (64 -> 1) in FP32 from those registers.
// The numerics are those of the mma.sync path (tlq_mlp.cuh) and of the CPU
// oracle: BF16 weights of layers 2-3 and BF16 activations fed to them, FP32
// accumulation, FP32 input and output layers.
//
// Operand layout: both operands are K-major without swizzling, in 8 x 8
// "core matrices" of BF16 (8 rows of 16 contiguous bytes, 128 bytes each):
// element (r, k) of an R x 64 matrix lives at byte
//   ((r / 8) * 8 + k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2,
// so core matrices adjacent in K are 128 bytes apart (the descriptor's
// leading-dimension byte offset) and adjacent 8-row groups 1024 bytes (its
// stride-dimension byte offset); the k-th K=16 slice starts 256 k bytes in.
#pragma once

#include <cuda_bf16.h>

#include <cstdint>

#include "tlq_device.cuh"
#include "tlq_mlp.cuh"

namespace tlq {
namespace umma {

constexpr int ROWS = 128;        // cells per tile = threads per block = MMA M
constexpr uint32_t TMEM_COLS = 64;  // FP32 accumulator columns (MMA N)
constexpr long long MMA_WAIT_LIMIT = 1LL << 22;  // mbarrier polls before giving up

struct alignas(128) Smem {
  __nv_bfloat16 a[ROWS * mlp::HID];       // activations of the tile (A operand), 16 KB
  __nv_bfloat16 w2[mlp::HID * mlp::HID];  // layer 2 weights, N x K (B operand), 8 KB
  __nv_bfloat16 w3[mlp::HID * mlp::HID];  // layer 3 weights, 8 KB
  float w1[mlp::HID][4];                  // layer 1, FP32 (in padded 3 -> 4)
  float w4[mlp::HID], b1[mlp::HID], b2[mlp::HID], b3[mlp::HID];
  float b4;
  uint64_t bar;   // MMA completion
  uint32_t tmem;  // TMEM address from tcgen05.alloc
  int failed;     // an MMA wait ran out (block-wide)
};

__device__ __forceinline__ uint32_t core_offset(int r, int k) {
  return (uint32_t)(((r >> 3) * 8 + (k >> 3)) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// Shared-memory matrix descriptor (tcgen05): start address, leading- and
// stride-dimension byte offsets (all in 16-byte units), descriptor version 1
// at bit 46, base offset 0, no swizzling.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)(128u >> 4) << 16;   // K-adjacent core matrices
  d |= (uint64_t)(1024u >> 4) << 32;  // adjacent 8-row groups
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor of kind::f16: D FP32 (bits 4-5 = 1), A and B BF16
// (bits 7-9 = 1, 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 at bit
// 17, M >> 4 at bit 24.
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(mlp::HID >> 3) << 17) |
                           ((uint32_t)(ROWS >> 4) << 24);

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// D[tmem] (+)= A x B^T over one K=16 slice.
__device__ __forceinline__ void mma(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, bool accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(IDESC), "r"((uint32_t)accumulate)
      : "memory");
}

__device__ __forceinline__ void commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// 32 consecutive FP32 columns of this thread's TMEM lane.
__device__ __forceinline__ void ld32(uint32_t taddr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int q = 0; q < 32; ++q) v[q] = __uint_as_float(r[q]);
}

// The block's copy of a network image (tlq_mlp.cuh's SmemWeights, formed
// once in device memory): layers 2-3 rearranged into core matrices with
// 16-byte moves (a padded row of the image holds 9 chunks of 8 BF16), the
// FP32 parts copied.  All threads.
__device__ __forceinline__ void load_weights(const mlp::SmemWeights* __restrict__ img, Smem& s) {
  constexpr int CH = mlp::HID / 8;  // 16-byte chunks per row
  for (int q = threadIdx.x; q < 2 * mlp::HID * CH; q += blockDim.x) {
    const int m = q / (mlp::HID * CH), rem = q % (mlp::HID * CH), n = rem / CH, c = rem % CH;
    const __nv_bfloat16* src = m == 0 ? &img->w2[n][8 * c] : &img->w3[n][8 * c];
    const uint4 v = __ldg(reinterpret_cast<const uint4*>(src));
    unsigned char* dst = reinterpret_cast<unsigned char*>(m == 0 ? s.w2 : s.w3) + core_offset(n, 8 * c);
    *reinterpret_cast<uint4*>(dst) = v;
  }
  for (int q = threadIdx.x; q < mlp::HID; q += blockDim.x) {
    *reinterpret_cast<float4*>(s.w1[q]) = __ldg(reinterpret_cast<const float4*>(img->w1[q]));
    s.w4[q] = img->w4[q];
    s.b1[q] = img->b1[q];
    s.b2[q] = img->b2[q];
    s.b3[q] = img->b3[q];
  }
  if (threadIdx.x == 0) s.b4 = img->b4;
}

// The same from FP32 master parameters (packed as tlq_mlp.cuh's OFF_*): the
// standalone inference entry point.  All threads.
__device__ __forceinline__ void load_weights_fp32(const float* __restrict__ P, Smem& s) {
  unsigned char* w2 = reinterpret_cast<unsigned char*>(s.w2);
  unsigned char* w3 = reinterpret_cast<unsigned char*>(s.w3);
  for (int q = threadIdx.x; q < mlp::HID * mlp::HID; q += blockDim.x) {
    const int n = q / mlp::HID, k = q % mlp::HID;
    *reinterpret_cast<__nv_bfloat16*>(w2 + core_offset(n, k)) = __float2bfloat16_rn(P[mlp::OFF_W2 + q]);
    *reinterpret_cast<__nv_bfloat16*>(w3 + core_offset(n, k)) = __float2bfloat16_rn(P[mlp::OFF_W3 + q]);
  }
  for (int q = threadIdx.x; q < mlp::HID; q += blockDim.x) {
    for (int f = 0; f < 4; ++f) s.w1[q][f] = f < mlp::IN ? P[mlp::OFF_W1 + q * mlp::IN + f] : 0.0f;
    s.w4[q] = P[mlp::OFF_W4 + q];
    s.b1[q] = P[mlp::OFF_B1 + q];
    s.b2[q] = P[mlp::OFF_B2 + q];
    s.b3[q] = P[mlp::OFF_B3 + q];
  }
  if (threadIdx.x == 0) s.b4 = P[mlp::OFF_B4];
}

// After a wait that ran out (failed): thread 0 waits once more, bounded, for
// the MMA it issued, so that tear-down does not free TMEM under it.
__device__ __forceinline__ void drain(Smem& s, uint32_t phase) {
  if (threadIdx.x == 0) mbar_wait_bounded(&s.bar, phase ^ 1u, MMA_WAIT_LIMIT);
  __syncthreads();
}

// Set-up (all threads): warp 0 allocates the TMEM columns, thread 0
// initialises the mbarrier.
__device__ __forceinline__ void setup(Smem& s) {
  if (threadIdx.x < 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&s.tmem)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (threadIdx.x == 0) {
    mbar_init(&s.bar, 1);
    s.failed = 0;
    fence_mbar_init();
  }
  fence_before();
  __syncthreads();
  fence_after();
}

// Tear-down (all threads): warp 0 frees the TMEM columns.  Every MMA this
// block issued has completed (its waits succeeded) or was waited for with a
// bound (failed).
__device__ __forceinline__ void teardown(Smem& s) {
  fence_before();
  __syncthreads();
  fence_after();
  if (threadIdx.x < 32)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(s.tmem), "r"(TMEM_COLS) : "memory");
}

// Eight activations (SiLU applied) of this thread's row, columns
// 8c..8c+7, as BF16 into the A operand (one 16-byte store).
__device__ __forceinline__ void store_chunk(Smem& s, int r, int c, const float* h8) {
  uint4 v;
  v.x = mlp::pack_bf16(h8[0], h8[1]);
  v.y = mlp::pack_bf16(h8[2], h8[3]);
  v.z = mlp::pack_bf16(h8[4], h8[5]);
  v.w = mlp::pack_bf16(h8[6], h8[7]);
  *reinterpret_cast<uint4*>(reinterpret_cast<unsigned char*>(s.a) + core_offset(r, 8 * c)) = v;
}

// One hidden layer on the tensor cores: D = A x W^T (64 columns of TMEM),
// issued by thread 0 after every thread's row of A is in shared memory;
// every thread waits for its completion (bounded; the outcome is agreed
// block-wide).  Returns false when the wait ran out.
__device__ __forceinline__ bool layer_mma(Smem& s, const __nv_bfloat16* w, uint32_t& phase) {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // A's stores -> the tensor core's view
  fence_before();
  __syncthreads();
  fence_after();
  if (threadIdx.x == 0) {
    const uint32_t a0 = smem_u32(s.a), b0 = smem_u32(w);
#pragma unroll
    for (int kk = 0; kk < mlp::HID / 16; ++kk) mma(s.tmem, smem_desc(a0 + 256u * kk), smem_desc(b0 + 256u * kk), kk > 0);
    commit(&s.bar);
  }
  const bool ok = mbar_wait_bounded(&s.bar, phase, MMA_WAIT_LIMIT);
  phase ^= 1u;
  fence_after();
  return !__syncthreads_or(!ok);
}

// The network on this thread's cell: features x (normalised) -> y.  All
// 128 threads of the block call it together.  The row is streamed in
// pieces (8 columns of layer 1, 32 TMEM columns of layers 2-3), so that a
// thread never holds all 64 activations.  Returns false (and the block
// stops using the tensor cores) when an MMA wait ran out.
__device__ __forceinline__ bool forward(Smem& s, const float* x, float& y, uint32_t& phase) {
  const int r = threadIdx.x;
#pragma unroll
  for (int c = 0; c < mlp::HID / 8; ++c) {
    float h8[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const float4 w = *reinterpret_cast<const float4*>(s.w1[8 * c + q]);
      h8[q] = mlp::silu_f(s.b1[8 * c + q] + w.x * x[0] + w.y * x[1] + w.z * x[2]);
    }
    store_chunk(s, r, c, h8);
  }
  const uint32_t lane_base = s.tmem + ((uint32_t)(threadIdx.x & ~31u) << 16);
  if (!layer_mma(s, s.w2, phase)) return false;
  // layer 2's activations replace layer 1's in A (the MMA has consumed them)
#pragma unroll
  for (int half = 0; half < 2; ++half) {
    float v[32];
    ld32(lane_base + 32u * half, v);
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      float h8[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) h8[q] = mlp::silu_f(v[8 * c + q] + s.b2[32 * half + 8 * c + q]);
      store_chunk(s, r, 4 * half + c, h8);
    }
  }
  if (!layer_mma(s, s.w3, phase)) return false;
  float acc = 0.0f;
#pragma unroll
  for (int half = 0; half < 2; ++half) {
    float v[32];
    ld32(lane_base + 32u * half, v);
#pragma unroll
    for (int q = 0; q < 32; ++q) acc += s.w4[32 * half + q] * mlp::silu_f(v[q] + s.b3[32 * half + q]);
  }
  y = s.b4 + acc;
  return true;
}

}  // namespace umma
}  // namespace tlq
