// Device code of the occluder-proposal network shared by the training kernels
// (mlp.cu) and the fused inference kernel: mma.sync / ldmatrix wrappers, the
// activation, and fused_forward_kernel.
//
// fused_forward_kernel evaluates the whole network for 16 rows per warp
// without leaving the SM: the weights (bf16, ~82 KB) are staged once per
// block in shared memory, the input features of a 16-row tile are staged per
// warp, and each layer's output stays in registers. The m16n8k16 accumulator
// layout (row g = lane / 4, columns 2t, 2t + 1 with t = lane % 4, rows g and
// g + 8) is the A-fragment layout of the next layer's 16-column K slice, so a
// finished pair of 8-column output tiles is biased, passed through GELU,
// rounded to bf16 and packed straight into the next layer's A operand. The
// rounding points (bf16 inputs, weights and hidden activations, fp32
// accumulation in ascending K slices, bias after the product) are those of
// the unfused training forward.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "mlp.h"

namespace qbc {
namespace mlp {

__device__ __forceinline__ float gelu_f(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void ldsm_x4(uint32_t addr, uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(addr));
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t*>(&v);
}

constexpr int kFusedWarps = 8;
constexpr int kFusedThreads = kFusedWarps * 32;
constexpr int kLdIn = kIn + 8;      // padded rows (bytes a multiple of 16, ldmatrix conflict-free)
constexpr int kLdH = kHidden + 8;
constexpr int kOutRows = 8;         // output rows of the last layer computed (0..3 used)

struct FusedSmem {
  __nv_bfloat16 w1[kHidden * kLdIn];
  __nv_bfloat16 w2[kHidden * kLdH];
  __nv_bfloat16 w3[kHidden * kLdH];
  __nv_bfloat16 w4[kOutRows * kLdH];
  float bias[3 * kHidden + kOutRows];
  __nv_bfloat16 x[kFusedWarps][16 * kLdIn];
  float out[kFusedWarps][16 * kOutUsed];
};

// Weights and biases of one network (device pointers, [out][in] rows).
struct FusedParams {
  const __nv_bfloat16* w[4];
  const float* b[4];
};

// One hidden layer for the warp's 16 rows: a (KS slices of the input) ->
// a (8 slices of GELU(W x + b), bf16).
template <int KS>
__device__ __forceinline__ void fused_hidden_layer(const __nv_bfloat16* W, int ld, const float* bias,
                                                   uint32_t (&a)[8][4], int lane) {
  uint32_t o[8][4];
  const int t = lane & 3;
#pragma unroll
  for (int np = 0; np < 8; ++np) {
    float c0[4] = {0.0f, 0.0f, 0.0f, 0.0f}, c1[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    const int row = np * 16 + (lane & 7) + ((lane >> 4) << 3);
#pragma unroll
    for (int kk = 0; kk < KS; ++kk) {
      uint32_t b0, b1, b2, b3;
      ldsm_x4(smem_u32(W + row * ld + kk * 16 + ((lane >> 3) & 1) * 8), b0, b1, b2, b3);
      mma_bf16(c0, a[kk], b0, b1);
      mma_bf16(c1, a[kk], b2, b3);
    }
    const int n0 = np * 16 + 2 * t, n1 = n0 + 8;
    o[np][0] = pack_bf16(gelu_f(c0[0] + bias[n0]), gelu_f(c0[1] + bias[n0 + 1]));
    o[np][1] = pack_bf16(gelu_f(c0[2] + bias[n0]), gelu_f(c0[3] + bias[n0 + 1]));
    o[np][2] = pack_bf16(gelu_f(c1[0] + bias[n1]), gelu_f(c1[1] + bias[n1 + 1]));
    o[np][3] = pack_bf16(gelu_f(c1[2] + bias[n1]), gelu_f(c1[3] + bias[n1 + 1]));
  }
#pragma unroll
  for (int k = 0; k < 8; ++k)
#pragma unroll
    for (int r = 0; r < 4; ++r) a[k][r] = o[k][r];
}

// Src: rows() (device-side row count), load(r0, n, x, lane) writing the
// features of rows r0 .. r0 + 15 as bf16 rows of kLdIn into x (rows >= n
// zero; all 32 lanes call it), store(r, o) with o the kOutUsed outputs of
// row r (called by one lane per row).
template <class Src>
__global__ void __launch_bounds__(kFusedThreads, 2) fused_forward_kernel(const FusedParams p, const Src src) {
  extern __shared__ __align__(16) unsigned char fused_smem_raw[];
  FusedSmem& S = *reinterpret_cast<FusedSmem*>(fused_smem_raw);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

  // stage the weights in 16-byte vectors, biases as floats
  {
    constexpr int v1 = kIn / 8, vh = kHidden / 8;
    for (int e = tid; e < kHidden * v1; e += kFusedThreads) {
      const int r = e / v1, c = e % v1;
      *reinterpret_cast<uint4*>(&S.w1[r * kLdIn + c * 8]) = reinterpret_cast<const uint4*>(p.w[0])[r * v1 + c];
    }
    for (int e = tid; e < kHidden * vh; e += kFusedThreads) {
      const int r = e / vh, c = e % vh;
      *reinterpret_cast<uint4*>(&S.w2[r * kLdH + c * 8]) = reinterpret_cast<const uint4*>(p.w[1])[r * vh + c];
      *reinterpret_cast<uint4*>(&S.w3[r * kLdH + c * 8]) = reinterpret_cast<const uint4*>(p.w[2])[r * vh + c];
    }
    for (int e = tid; e < kOutRows * vh; e += kFusedThreads) {
      const int r = e / vh, c = e % vh;
      *reinterpret_cast<uint4*>(&S.w4[r * kLdH + c * 8]) = reinterpret_cast<const uint4*>(p.w[3])[r * vh + c];
    }
    for (int e = tid; e < 3 * kHidden + kOutRows; e += kFusedThreads)
      S.bias[e] = e < 3 * kHidden ? p.b[e / kHidden][e % kHidden] : p.b[3][e - 3 * kHidden];
  }
  __syncthreads();

  const uint32_t rows = src.rows();
  const uint32_t tiles = (rows + 15u) / 16u;
  const int g = lane >> 2, t = lane & 3;
  __nv_bfloat16* x = S.x[warp];
  float* out = S.out[warp];
  for (uint32_t tile = blockIdx.x * kFusedWarps + warp; tile < tiles; tile += gridDim.x * kFusedWarps) {
    const uint32_t r0 = tile * 16u;
    __syncwarp();
    src.load(r0, min(16u, rows - r0), x, lane);
    __syncwarp();
    uint32_t a[8][4];
#pragma unroll
    for (int kk = 0; kk < kIn / 16; ++kk)
      ldsm_x4(smem_u32(x + (lane & 15) * kLdIn + kk * 16 + (lane >> 4) * 8), a[kk][0], a[kk][1], a[kk][2],
              a[kk][3]);
    fused_hidden_layer<kIn / 16>(S.w1, kLdIn, S.bias, a, lane);
    fused_hidden_layer<kHidden / 16>(S.w2, kLdH, S.bias + kHidden, a, lane);
    fused_hidden_layer<kHidden / 16>(S.w3, kLdH, S.bias + 2 * kHidden, a, lane);
    float c[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int kk = 0; kk < kHidden / 16; kk += 2) {
      uint32_t b0, b1, b2, b3;
      ldsm_x4(smem_u32(S.w4 + (lane & 7) * kLdH + kk * 16 + (lane >> 3) * 8), b0, b1, b2, b3);
      mma_bf16(c, a[kk], b0, b1);
      mma_bf16(c, a[kk + 1], b2, b3);
    }
    if (t < kOutUsed / 2) {
      const float* b4 = S.bias + 3 * kHidden;
      out[g * kOutUsed + 2 * t] = c[0] + b4[2 * t];
      out[g * kOutUsed + 2 * t + 1] = c[1] + b4[2 * t + 1];
      out[(g + 8) * kOutUsed + 2 * t] = c[2] + b4[2 * t];
      out[(g + 8) * kOutUsed + 2 * t + 1] = c[3] + b4[2 * t + 1];
    }
    __syncwarp();
    if (lane < 16 && r0 + lane < rows) src.store(r0 + lane, out + lane * kOutUsed);
  }
}

}  // namespace mlp
}  // namespace qbc
