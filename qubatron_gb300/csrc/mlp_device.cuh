// Device code of the occluder-proposal network shared by the training kernels
// (mlp.cu) and the inference kernel: the activation, bf16 packing, and
// umma_forward_kernel, the whole network on the tcgen05 tensor cores.

#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "mlp.h"
#include "qbc_internal.h"
#include "umma.cuh"

namespace qbc {
namespace mlp {

__device__ __forceinline__ float gelu_f(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t*>(&v);
}

constexpr int kLdIn = kIn + 8;  // padded feature rows a Src loads (bytes a multiple of 16)

// ---- fused inference on the 5th-generation tensor cores (tcgen05) ----
//
// umma_forward_kernel evaluates the whole network for 128 rows per tile on
// one SM: the four weight matrices (bf16, 80 KB) are staged once per block in
// shared memory in the K-major core-matrix layout (umma.cuh); per tile the
// features go to shared memory in the same layout, and each layer is one
// chain of tcgen05.mma (M = 128, N = 128, or 16 for the output layer, K = 16
// per instruction) issued by one thread into a 128-column fp32 accumulator in
// tensor memory. The 8 warps then read the accumulator (warp w: rows 32 (w %
// 4) .. + 31, columns 64 (w / 4) .. + 63), add the bias, apply GELU, round
// to bf16 and write the next layer's A operand back to shared memory. The
// rounding points are those of the training forward: bf16 inputs, weights
// and hidden activations, fp32 accumulation, bias after the product.
constexpr int kUmmaRows = 128;
constexpr int kUmmaWarps = 8;
constexpr int kUmmaThreads = kUmmaWarps * 32;
constexpr uint32_t kUmmaTmemCols = 256;        // 128 used; power of two
constexpr uint32_t kUmmaWaitLimit = 1u << 24;  // polls (~1 s) before a wait gives up

struct UmmaSmem {
  // operand regions, each a multiple of 1024 bytes from a 1024-aligned base
  __nv_bfloat16 w1[kHidden * kIn];
  __nv_bfloat16 w2[kHidden * kHidden];
  __nv_bfloat16 w3[kHidden * kHidden];
  __nv_bfloat16 w4[kOutPad * kHidden];
  __nv_bfloat16 x[kUmmaRows * kIn];
  __nv_bfloat16 h[kUmmaRows * kHidden];
  __nv_bfloat16 stage[kUmmaWarps][16 * kLdIn];
  float bias[3 * kHidden + kOutPad];
  uint64_t bar;
  uint32_t tmem;
  uint32_t fault;
};
constexpr size_t kUmmaSmemBytes = sizeof(UmmaSmem) + 1024;  // + alignment slack

// Weights and biases of one network (device pointers, [out][in] rows).
struct FusedParams {
  const __nv_bfloat16* w[4];
  const float* b[4];
};

// Rows x cols (bf16, row-major, 16-byte aligned rows) -> core layout.
__device__ __forceinline__ void stage_matrix(__nv_bfloat16* dst, const __nv_bfloat16* src, int rows, int cols,
                                             int tid, int nthreads) {
  const int vec = cols / 8;
  for (int e = tid; e < rows * vec; e += nthreads) {
    const int r = e / vec, c = e % vec;
    const uint4 v = reinterpret_cast<const uint4*>(src)[(size_t)r * vec + c];
    *reinterpret_cast<uint4*>(reinterpret_cast<char*>(dst) + umma::core_offset(r, 8 * c, cols)) = v;
  }
}

// One layer's MMA chain: D[128 x N] = A[128 x K] * B[N x K]^T (both K-major).
__device__ __forceinline__ void issue_layer(uint32_t tmem, const __nv_bfloat16* a, const __nv_bfloat16* b, int K,
                                            int N) {
  const uint32_t sa = umma::smem_addr(a), sb = umma::smem_addr(b);
  const uint32_t idesc = umma::idesc_bf16(kUmmaRows, N);
  for (int k0 = 0; k0 < K; k0 += 16)
    umma::mma_bf16(tmem, umma::slice_desc(sa, k0, K), umma::slice_desc(sb, k0, K), idesc, k0 > 0);
}

// Hidden-layer epilogue: accumulator -> GELU(acc + bias) as bf16 into h.
__device__ __forceinline__ void hidden_epilogue(uint32_t tmem, const float* bias, __nv_bfloat16* h, int warp,
                                                int lane) {
  const int q = warp & 3, half = warp >> 2;
  const int row = 32 * q + lane;
  float v[2][32];
  umma::tmem_ld32(tmem + ((uint32_t)(32 * q) << 16) + 64 * half, v[0]);
  umma::tmem_ld32(tmem + ((uint32_t)(32 * q) << 16) + 64 * half + 32, v[1]);
  umma::tmem_ld_wait();
#pragma unroll
  for (int j = 0; j < 2; ++j) {
#pragma unroll
    for (int g = 0; g < 4; ++g) {
      const int c0 = 64 * half + 32 * j + 8 * g;
      uint4 o;
      o.x = pack_bf16(gelu_f(v[j][8 * g + 0] + bias[c0 + 0]), gelu_f(v[j][8 * g + 1] + bias[c0 + 1]));
      o.y = pack_bf16(gelu_f(v[j][8 * g + 2] + bias[c0 + 2]), gelu_f(v[j][8 * g + 3] + bias[c0 + 3]));
      o.z = pack_bf16(gelu_f(v[j][8 * g + 4] + bias[c0 + 4]), gelu_f(v[j][8 * g + 5] + bias[c0 + 5]));
      o.w = pack_bf16(gelu_f(v[j][8 * g + 6] + bias[c0 + 6]), gelu_f(v[j][8 * g + 7] + bias[c0 + 7]));
      *reinterpret_cast<uint4*>(reinterpret_cast<char*>(h) + umma::core_offset(row, c0, kHidden)) = o;
    }
  }
}

// Src: rows() (device-side row count), load(r0, n, x, lane) writing the
// features of rows r0 .. r0 + 15 as bf16 rows of kLdIn into x (rows >= n
// zero; all 32 lanes call it), store(r, o) with o the kOutUsed outputs of
// row r. err receives kErrMmaTimeout if a tensor-core wait gave up (the
// block then stops, frees its tensor memory and returns).
template <class Src>
__global__ void __launch_bounds__(kUmmaThreads, 1) umma_forward_kernel(const FusedParams p, const Src src,
                                                                       unsigned* err) {
  extern __shared__ unsigned char umma_smem_raw[];
  UmmaSmem& S = *reinterpret_cast<UmmaSmem*>(
      (reinterpret_cast<uintptr_t>(umma_smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

  stage_matrix(S.w1, p.w[0], kHidden, kIn, tid, kUmmaThreads);
  stage_matrix(S.w2, p.w[1], kHidden, kHidden, tid, kUmmaThreads);
  stage_matrix(S.w3, p.w[2], kHidden, kHidden, tid, kUmmaThreads);
  stage_matrix(S.w4, p.w[3], kOutPad, kHidden, tid, kUmmaThreads);
  for (int e = tid; e < 3 * kHidden + kOutPad; e += kUmmaThreads)
    S.bias[e] = e < 3 * kHidden ? p.b[e / kHidden][e % kHidden] : p.b[3][e - 3 * kHidden];
  if (tid == 0) {
    S.fault = 0u;
    umma::mbar_init(&S.bar, 1);
  }
  if (warp == 0) {
    umma::tmem_alloc(&S.tmem, kUmmaTmemCols);
    umma::tmem_relinquish();
  }
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = S.tmem;
  uint32_t phase = 0;

  const uint32_t rows = src.rows();
  const uint32_t tiles = (rows + kUmmaRows - 1) / kUmmaRows;
  __nv_bfloat16* stage = S.stage[warp];
  for (uint32_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    // features of the tile's rows: warp w loads rows 16 w .. 16 w + 15
    const uint32_t r0 = tile * kUmmaRows + 16u * warp;
    const uint32_t n = r0 < rows ? min(16u, rows - r0) : 0u;
    __syncwarp();
    src.load(r0, n, stage, lane);
    __syncwarp();
    for (int e = lane; e < 16 * (kIn / 8); e += 32) {
      const int r = e / (kIn / 8), c = e % (kIn / 8);
      *reinterpret_cast<uint4*>(reinterpret_cast<char*>(S.x) + umma::core_offset(16 * warp + r, 8 * c, kIn)) =
          *reinterpret_cast<const uint4*>(stage + r * kLdIn + 8 * c);
    }
    bool stop = false;
    // four layers: MMA chain by thread 0, then the epilogue by all warps
    for (int layer = 0; layer < 4 && !stop; ++layer) {
      umma::fence_smem_to_async();
      umma::fence_before_sync();
      __syncthreads();
      if (tid == 0) {
        umma::fence_after_sync();
        if (layer == 0) issue_layer(tmem, S.x, S.w1, kIn, kHidden);
        else if (layer == 1) issue_layer(tmem, S.h, S.w2, kHidden, kHidden);
        else if (layer == 2) issue_layer(tmem, S.h, S.w3, kHidden, kHidden);
        else issue_layer(tmem, S.h, S.w4, kHidden, kOutPad);
        umma::commit(&S.bar);
      }
      if (!umma::mbar_wait(&S.bar, phase, kUmmaWaitLimit)) atomicOr(&S.fault, 1u);
      umma::fence_after_sync();
      __syncthreads();
      if (S.fault) {
        stop = true;
        break;
      }
      phase ^= 1u;
      if (layer < 3) {
        hidden_epilogue(tmem, S.bias + layer * kHidden, S.h, warp, lane);
      } else if (warp < 4) {
        float v[32];
        umma::tmem_ld32(tmem + ((uint32_t)(32 * warp) << 16), v);
        umma::tmem_ld_wait();
        const uint32_t r = tile * kUmmaRows + 32u * warp + lane;
        if (r < rows) {
          float o[kOutUsed];
#pragma unroll
          for (int k = 0; k < kOutUsed; ++k) o[k] = v[k] + S.bias[3 * kHidden + k];
          src.store(r, o);
        }
      }
    }
    if (stop) break;
    umma::fence_before_sync();  // the next tile's MMAs overwrite the accumulator
  }
  __syncthreads();
  if (S.fault) {
    if (tid == 0) {
      atomicOr(err, kErrMmaTimeout);
      umma::mbar_wait(&S.bar, phase, kUmmaWaitLimit);  // the MMAs in flight
    }
    __syncthreads();
  }
  umma::fence_after_sync();
  if (warp == 0) umma::tmem_dealloc(tmem, kUmmaTmemCols);
}

}  // namespace mlp
}  // namespace qbc
