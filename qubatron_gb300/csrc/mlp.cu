// Occluder-proposal network: 48 -> 128 -> 128 -> 128 -> 16 (3 used), GELU,
// BF16 weights and activations on the tensor cores with FP32 accumulation,
// trained on the GPU with hand-written forward, backward and Adam kernels.
//
// Every matrix product goes through one kernel, gemm_kernel, on the tcgen05
// tensor cores: a 128 x 64 output tile per block of 4 warps in a tensor-memory
// accumulator, operands staged in shared memory in 32-deep K slices (two
// stages, transposed as the product needs), bf16 x bf16 -> f32. The epilogue
// reads the accumulator with tcgen05.ld, adds the bias, applies GELU, stores
// the pre-activation (for backward) and the bf16 activation, or accumulates
// into an fp32 result with atomics (weight gradients, where the reduction
// runs over the batch and is split across blocks).

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "mlp.h"
#include "mlp_device.cuh"
#include "qbc_internal.h"

using qbc::fail;

namespace qbc {
namespace mlp {

// kernels launched by this thread (the context adds the difference to its
// launch count)
thread_local int64_t g_launches = 0;
int64_t launches() { return g_launches; }

namespace {

using bf16 = __nv_bfloat16;

// GEMM tiles on the tcgen05 tensor cores: a block computes a 128 (M) x 64 (N)
// tile of C into a 64-column fp32 accumulator in tensor memory, with K in
// slices of 32 staged by the block's threads into one of two shared-memory
// stages (K-major core-matrix layout, umma.cuh; op(A) and op(B) transposed
// while staging) while the previous slice's MMAs run.
constexpr int kTileM = 128;
constexpr int kTileN = 64;
constexpr int kKs = 32;
constexpr int kGemmThreads = 128;
constexpr uint32_t kGemmTmemCols = 64;
// dynamic shared memory per block: two stages of A (8 KB) and B (4 KB), the
// barriers, and headroom that keeps at most 7 blocks on an SM (7 x 64 of its
// 512 tensor-memory columns)
constexpr int kGemmSmemBytes = 32 * 1024;

struct GemmSmem {
  bf16 a[2][kTileM * kKs];
  bf16 b[2][kTileN * kKs];
  uint64_t bar[2];
  uint64_t done;
  uint32_t tmem;
  uint32_t fault;
};
static_assert(sizeof(GemmSmem) + 1024 <= kGemmSmemBytes, "gemm shared memory");

struct Epi {
  float* C;         // fp32 output (or atomic accumulator)
  int ldc;
  bf16* Cb;         // bf16 output (activation)
  int ldcb;
  float* Z;         // fp32 pre-activation copy
  int ldz;
  const float* bias;
  int gelu;
  int atomic;
  unsigned* err;    // kErrMmaTimeout when a tensor-core wait gave up
};

__device__ __forceinline__ float gelu_grad(float x) {
  const float cdf = 0.5f * (1.0f + erff(x * 0.70710678118654752f));
  const float pdf = 0.39894228040143268f * expf(-0.5f * x * x);
  return cdf + x * pdf;
}

// C[M x N] = op(A)[M x K] * op(B)[K x N]. A is M x K row-major (TA false) or
// K x M row-major (TA true); B is K x N row-major (TB false) or N x K
// row-major (TB true). Block z handles K rows [z * kchunk, (z + 1) * kchunk).
template <bool TA, bool TB>
__global__ void __launch_bounds__(kGemmThreads) gemm_kernel(const bf16* __restrict__ A, int lda,
                                                            const bf16* __restrict__ B, int ldb, int M, int N, int K,
                                                            int kchunk, Epi epi) {
  extern __shared__ unsigned char gemm_smem_raw[];
  GemmSmem& S = *reinterpret_cast<GemmSmem*>((reinterpret_cast<uintptr_t>(gemm_smem_raw) + 1023) &
                                             ~static_cast<uintptr_t>(1023));
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int m0 = blockIdx.y * kTileM, n0 = blockIdx.x * kTileN;
  const int kb = blockIdx.z * kchunk, ke = min(K, kb + kchunk);
  if (tid == 0) {
    S.fault = 0u;
    umma::mbar_init(&S.bar[0], 1);
    umma::mbar_init(&S.bar[1], 1);
    umma::mbar_init(&S.done, 1);
  }
  if (warp == 0) {
    umma::tmem_alloc(&S.tmem, kGemmTmemCols);
    umma::tmem_relinquish();
  }
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = S.tmem;
  const uint32_t idesc = umma::idesc_bf16(kTileM, kTileN);
  const bf16 zero = __float2bfloat16(0.0f);
  uint32_t ph[2] = {0u, 0u};
  int it = 0;
  for (int k0 = kb; k0 < ke; k0 += kKs, ++it) {
    const int st = it & 1;
    if (it >= 2) {  // the MMAs of slice it - 2 have read this stage
      if (!umma::mbar_wait(&S.bar[st], ph[st], kUmmaWaitLimit)) atomicOr(&S.fault, 1u);
      ph[st] ^= 1u;
    }
    // stage op(A)[m0.., k0..] and op(B)[k0.., n0..] (consecutive threads
    // along each operand's contiguous dimension)
    char* as = reinterpret_cast<char*>(S.a[st]);
    char* bs = reinterpret_cast<char*>(S.b[st]);
    for (int e = tid; e < kTileM * kKs; e += kGemmThreads) {
      const int r = TA ? e % kTileM : e / kKs, c = TA ? e / kTileM : e % kKs;  // r: m, c: k
      const int m = m0 + r, k = k0 + c;
      bf16 v = zero;
      if (m < M && k < ke) v = TA ? A[(size_t)k * lda + m] : A[(size_t)m * lda + k];
      *reinterpret_cast<bf16*>(as + umma::core_offset(r, c, kKs)) = v;
    }
    for (int e = tid; e < kTileN * kKs; e += kGemmThreads) {
      const int r = TB ? e / kKs : e % kTileN, c = TB ? e % kKs : e / kTileN;  // r: n, c: k
      const int n = n0 + r, k = k0 + c;
      bf16 v = zero;
      if (n < N && k < ke) v = TB ? B[(size_t)n * ldb + k] : B[(size_t)k * ldb + n];
      *reinterpret_cast<bf16*>(bs + umma::core_offset(r, c, kKs)) = v;
    }
    umma::fence_smem_to_async();
    umma::fence_before_sync();
    __syncthreads();
    if (S.fault) break;
    if (tid == 0) {
      umma::fence_after_sync();
      const uint32_t sa = umma::smem_addr(as), sb = umma::smem_addr(bs);
#pragma unroll
      for (int kk = 0; kk < kKs; kk += 16)
        umma::mma_bf16(tmem, umma::slice_desc(sa, kk, kKs), umma::slice_desc(sb, kk, kKs), idesc,
                       it > 0 || kk > 0);
      umma::commit(&S.bar[st]);
    }
  }
  // every MMA of this block done
  if (tid == 0) umma::commit(&S.done);
  if (!umma::mbar_wait(&S.done, 0, kUmmaWaitLimit)) atomicOr(&S.fault, 1u);
  umma::fence_after_sync();
  __syncthreads();
  if (S.fault) {
    if (tid == 0 && epi.err) atomicOr(epi.err, kErrMmaTimeout);
  } else {
    float v[2][32];
    umma::tmem_ld32(tmem + ((uint32_t)(32 * warp) << 16), v[0]);
    umma::tmem_ld32(tmem + ((uint32_t)(32 * warp) << 16) + 32, v[1]);
    umma::tmem_ld_wait();
    const int m = m0 + 32 * warp + lane;
    if (m < M) {
#pragma unroll
      for (int j = 0; j < kTileN; ++j) {
        const int n = n0 + j;
        if (n >= N) break;
        float x = it > 0 ? v[j >> 5][j & 31] : 0.0f;
        if (epi.atomic) {
          if (it > 0) atomicAdd(&epi.C[(size_t)m * epi.ldc + n], x);
          continue;
        }
        if (epi.bias) x += epi.bias[n];
        if (epi.Z) epi.Z[(size_t)m * epi.ldz + n] = x;
        if (epi.gelu) x = gelu_f(x);
        if (epi.C) epi.C[(size_t)m * epi.ldc + n] = x;
        if (epi.Cb) epi.Cb[(size_t)m * epi.ldcb + n] = __float2bfloat16(x);
      }
    }
  }
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  if (warp == 0) umma::tmem_dealloc(tmem, kGemmTmemCols);
}

template <bool TA, bool TB>
int gemm(const bf16* A, int lda, const bf16* B, int ldb, int64_t M, int N, int64_t K, const Epi& epi,
         cudaStream_t s, int64_t kchunk = 0) {
  if (M <= 0 || N <= 0 || K <= 0) return QBC_OK;
  if (kchunk <= 0) kchunk = K;
  kchunk = (kchunk + kKs - 1) / kKs * kKs;
  dim3 grid((unsigned)((N + kTileN - 1) / kTileN), (unsigned)((M + kTileM - 1) / kTileM),
            (unsigned)((K + kchunk - 1) / kchunk));
  if (grid.y > 65535u) return fail(QBC_E_ARG, "mlp gemm: %lld rows exceed one launch", (long long)M);
  static bool attr[4] = {false, false, false, false};
  const int v = (TA ? 1 : 0) + (TB ? 2 : 0);
  if (!attr[v]) {
    cudaError_t e = cudaFuncSetAttribute(gemm_kernel<TA, TB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         kGemmSmemBytes);
    if (e != cudaSuccess) return fail(QBC_E_CUDA, "mlp gemm attribute: %s", cudaGetErrorString(e));
    attr[v] = true;
  }
  gemm_kernel<TA, TB><<<grid, kGemmThreads, kGemmSmemBytes, s>>>(A, lda, B, ldb, (int)M, N, (int)K, (int)kchunk, epi);
  ++g_launches;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(QBC_E_CUDA, "mlp gemm launch: %s", cudaGetErrorString(e));
  return QBC_OK;
}

// ---- elementwise kernels ----

__global__ void to_bf16_kernel(const float* __restrict__ src, bf16* __restrict__ dst, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = __float2bfloat16(src[i]);
}

// Loss of the proposals o (first 3 of 16 columns) and its gradient (bf16,
// 16 columns). kind 1: the plain shadow walk found an occluder at t: the
// nearest output is pulled to t (winner takes all) and the others weakly.
// kind 0: the pixel was lit: every output is pushed past 1.1 (no proposal).
__global__ void loss_kernel(const float* __restrict__ o, const float* __restrict__ tlab,
                            const int8_t* __restrict__ kind, int64_t M, float scale, bf16* __restrict__ dO,
                            float* __restrict__ loss) {
  float local = 0.0f;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < M; i += (int64_t)gridDim.x * blockDim.x) {
    float g[kOutUsed] = {0.0f, 0.0f, 0.0f, 0.0f};
    const float* oi = o + i * kOutPad;
    if (kind[i] == 1) {
      const float t = tlab[i];
      int best = 0;
      float bd = fabsf(oi[0] - t);
      for (int k = 1; k < 3; ++k)
        if (fabsf(oi[k] - t) < bd) {
          bd = fabsf(oi[k] - t);
          best = k;
        }
      for (int k = 0; k < 3; ++k) {
        const float d = oi[k] - t;
        const float w = k == best ? 1.0f : 0.02f;
        local += w * d * d;
        g[k] = 2.0f * w * d;
      }
    } else if (kind[i] == 0) {
      for (int k = 0; k < 3; ++k) {
        const float d = 1.1f - oi[k];
        if (d > 0.0f) {
          local += 0.5f * d * d;
          g[k] = -d;
        }
      }
    }
    if (kind[i] == 0 || kind[i] == 1) {
      // occluded-or-not logit: weighted binary cross-entropy
      const float z = oi[kGate], y = kind[i] == 1 ? 1.0f : 0.0f;
      local += kGateWeight * (fmaxf(z, 0.0f) - y * z + log1pf(expf(-fabsf(z))));
      g[kGate] = kGateWeight * (1.0f / (1.0f + expf(-z)) - y);
    }
    for (int k = 0; k < kOutPad; ++k) dO[i * kOutPad + k] = __float2bfloat16(k < kOutUsed ? g[k] * scale : 0.0f);
  }
  for (int off = 16; off > 0; off >>= 1) local += __shfl_down_sync(0xFFFFFFFFu, local, off);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, local * scale);
}

// dZ = dA * GELU'(Z), in bf16 for the next product.
__global__ void gelu_back_kernel(const float* __restrict__ dA, const float* __restrict__ Z, int64_t n,
                                 bf16* __restrict__ dZ) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    dZ[i] = __float2bfloat16(dA[i] * gelu_grad(Z[i]));
}

// db[n] += sum over rows of dZ[:, n]
__global__ void bias_grad_kernel(const bf16* __restrict__ dZ, int64_t M, int N, float* __restrict__ db) {
  const int n = blockIdx.x;
  float s = 0.0f;
  for (int64_t i = threadIdx.x; i < M; i += blockDim.x) s += __bfloat162float(dZ[i * N + n]);
  for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xFFFFFFFFu, s, off);
  __shared__ float part[32];
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.0f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += part[w];
    db[n] += t;
  }
}

__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, int64_t n, float lr, float b1, float b2, float eps, float c1,
                            float c2) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    m[i] = b1 * m[i] + (1.0f - b1) * gi;
    v[i] = b2 * v[i] + (1.0f - b2) * gi * gi;
    p[i] -= lr * (m[i] / c1) / (sqrtf(v[i] / c2) + eps);
  }
}

int grid1(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 4096)); }

}  // namespace

// Parameter offsets (floats) in the master array: W1 b1 W2 b2 W3 b3 W4 b4,
// each W as [out][in].
int64_t param_offset(int layer, bool bias) {
  const int64_t w1 = (int64_t)kHidden * kIn, w2 = (int64_t)kHidden * kHidden, w4 = (int64_t)kOutPad * kHidden;
  const int64_t sizes[8] = {w1, kHidden, w2, kHidden, w2, kHidden, w4, kOutPad};
  int64_t off = 0;
  for (int k = 0; k < 2 * layer + (bias ? 1 : 0); ++k) off += sizes[k];
  return off;
}

int64_t param_count() { return param_offset(4, false); }

void Net::release() {
  cudaFree(master);
  cudaFree(wb);
  cudaFree(grad);
  cudaFree(m);
  cudaFree(v);
  cudaFree(work);
  master = grad = m = v = nullptr;
  wb = nullptr;
  work = nullptr;
  work_rows = 0;
  ready = false;
}

int Net::init(uint64_t seed, cudaStream_t s) {
  const int64_t n = param_count();
  if (!master) {
    cudaError_t e = cudaMalloc(&master, n * 4);
    if (e == cudaSuccess) e = cudaMalloc(&wb, n * 2);
    if (e == cudaSuccess) e = cudaMalloc(&grad, n * 4);
    if (e == cudaSuccess) e = cudaMalloc(&m, n * 4);
    if (e == cudaSuccess) e = cudaMalloc(&v, n * 4);
    if (e != cudaSuccess) return fail(QBC_E_NOMEM, "mlp parameters: %s", cudaGetErrorString(e));
  }
  // uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) weights from a seeded splitmix64,
  // zero biases; padding rows / columns zero
  std::vector<float> h(n, 0.0f);
  uint64_t st = seed * 0x9E3779B97F4A7C15ull + 77;
  auto u01 = [&]() {
    uint64_t z = (st += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
  };
  const int ins[4] = {kIn, kHidden, kHidden, kHidden}, outs[4] = {kHidden, kHidden, kHidden, kOutPad};
  const int used_in[4] = {kInUsed, kHidden, kHidden, kHidden}, used_out[4] = {kHidden, kHidden, kHidden, kOutUsed};
  for (int l = 0; l < 4; ++l) {
    const double a = 1.0 / std::sqrt((double)used_in[l]);
    float* W = h.data() + param_offset(l, false);
    for (int o = 0; o < outs[l]; ++o)
      for (int i = 0; i < ins[l]; ++i)
        W[o * ins[l] + i] = (o < used_out[l] && i < used_in[l]) ? (float)((2.0 * u01() - 1.0) * a) : 0.0f;
  }
  // output bias: start with "no proposal" (t past the hit)
  float* b4 = h.data() + param_offset(3, true);
  for (int o = 0; o < kOut; ++o) b4[o] = 1.5f;
  cudaError_t e = cudaMemcpyAsync(master, h.data(), n * 4, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(m, 0, n * 4, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(v, 0, n * 4, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return fail(QBC_E_CUDA, "mlp init: %s", cudaGetErrorString(e));
  step_count = 0;
  ready = true;
  return sync_weights(s);
}

int Net::set(const float* host, cudaStream_t s) {
  if (!master) {
    int rc = init(1, s);
    if (rc) return rc;
  }
  cudaError_t e = cudaMemcpyAsync(master, host, param_count() * 4, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return fail(QBC_E_CUDA, "mlp set: %s", cudaGetErrorString(e));
  ready = true;
  return sync_weights(s);
}

int Net::get(float* host, cudaStream_t s) const {
  if (!master) return fail(QBC_E_STATE, "mlp: no parameters");
  cudaError_t e = cudaMemcpyAsync(host, master, param_count() * 4, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return fail(QBC_E_CUDA, "mlp get: %s", cudaGetErrorString(e));
  return QBC_OK;
}

int Net::sync_weights(cudaStream_t s) {
  const int64_t n = param_count();
  to_bf16_kernel<<<grid1(n), 256, 0, s>>>(master, wb, n);
  ++g_launches;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(QBC_E_CUDA, "mlp weights: %s", cudaGetErrorString(e));
  return QBC_OK;
}

int Net::ensure_work(int64_t rows) {
  if (work_rows >= rows) return QBC_OK;
  cudaFree(work);
  work = nullptr;
  work_rows = 0;
  // per row: Z1..Z3 fp32, A1..A3 bf16, dA fp32, dZ bf16 (hidden wide), O fp32, dO bf16
  const size_t per = (size_t)3 * kHidden * 4 + 3 * kHidden * 2 + kHidden * 4 + kHidden * 2 + kOutPad * 4 + kOutPad * 2;
  cudaError_t e = cudaMalloc(&work, per * (size_t)rows + 1024);
  if (e != cudaSuccess) return fail(QBC_E_NOMEM, "mlp work buffers for %lld rows: %s", (long long)rows,
                                    cudaGetErrorString(e));
  work_rows = rows;
  return QBC_OK;
}

// Views into the work buffer for `rows` rows.
struct Bufs {
  float* Z[3];
  bf16* A[3];
  float* dA;
  bf16* dZ;
  float* O;
  bf16* dO;
};

static Bufs carve(char* base, int64_t rows) {
  Bufs b;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    char* p = base + off;
    off += (bytes + 255) & ~size_t(255);
    return p;
  };
  for (int l = 0; l < 3; ++l) b.Z[l] = (float*)take((size_t)rows * kHidden * 4);
  for (int l = 0; l < 3; ++l) b.A[l] = (bf16*)take((size_t)rows * kHidden * 2);
  b.dA = (float*)take((size_t)rows * kHidden * 4);
  b.dZ = (bf16*)take((size_t)rows * kHidden * 2);
  b.O = (float*)take((size_t)rows * kOutPad * 4);
  b.dO = (bf16*)take((size_t)rows * kOutPad * 2);
  return b;
}

int Net::forward(const bf16* X, int64_t rows, float* out, cudaStream_t s, bool keep) {
  if (!ready) return fail(QBC_E_STATE, "mlp: not initialised");
  const bf16* W[4];
  const float* bsv[4];
  for (int l = 0; l < 4; ++l) {
    W[l] = wb + param_offset(l, false);
    bsv[l] = master + param_offset(l, true);
  }
  const int64_t chunk = keep ? rows : std::min<int64_t>(rows, kChunkRows);
  int rc = ensure_work(chunk);
  if (rc) return rc;
  for (int64_t r0 = 0; r0 < rows; r0 += chunk) {
    const int64_t n = std::min(chunk, rows - r0);
    Bufs b = carve((char*)work, chunk);
    const bf16* in = X + r0 * kIn;
    int ld = kIn;
    for (int l = 0; l < 3; ++l) {
      Epi e{nullptr, 0, b.A[l], kHidden, keep ? b.Z[l] : nullptr, kHidden, bsv[l], 1, 0, err};
      rc = gemm<false, true>(in, ld, W[l], l == 0 ? kIn : kHidden, n, kHidden, l == 0 ? kIn : kHidden, e, s);
      if (rc) return rc;
      in = b.A[l];
      ld = kHidden;
    }
    Epi e{out + r0 * kOutPad, kOutPad, nullptr, 0, nullptr, 0, bsv[3], 0, 0, err};
    rc = gemm<false, true>(in, kHidden, W[3], kHidden, n, kOutPad, kHidden, e, s);
    if (rc) return rc;
  }
  return QBC_OK;
}

int Net::gradient(const bf16* X, const float* tlab, const int8_t* kind, int64_t rows, float* loss, cudaStream_t s) {
  int rc = ensure_work(rows);
  if (rc) return rc;
  Bufs b = carve((char*)work, rows);
  rc = forward(X, rows, b.O, s, true);
  if (rc) return rc;
  const int64_t n = param_count();
  if (cudaMemsetAsync(grad, 0, n * 4, s) != cudaSuccess || cudaMemsetAsync(loss, 0, 4, s) != cudaSuccess)
    return fail(QBC_E_CUDA, "mlp gradient: memset");
  const float scale = 1.0f / (float)rows;
  loss_kernel<<<grid1(rows), 256, 0, s>>>(b.O, tlab, kind, rows, scale, b.dO, loss);
  ++g_launches;
  const bf16* W[4];
  for (int l = 0; l < 4; ++l) W[l] = wb + param_offset(l, false);
  // weight gradients reduce over the batch: 256-row K chunks give the
  // product enough blocks (their partial sums meet in atomics)
  const int64_t kchunk = 256;
  // layer 4: dW4 = dO^T A3, db4 = sum dO, dA3 = dO W4
  {
    Epi e{grad + param_offset(3, false), kHidden, nullptr, 0, nullptr, 0, nullptr, 0, 1, err};
    rc = gemm<true, false>(b.dO, kOutPad, b.A[2], kHidden, kOutPad, kHidden, rows, e, s, kchunk);
    if (rc) return rc;
    bias_grad_kernel<<<kOutPad, 256, 0, s>>>(b.dO, rows, kOutPad, grad + param_offset(3, true));
    ++g_launches;
    Epi d{b.dA, kHidden, nullptr, 0, nullptr, 0, nullptr, 0, 0, err};
    rc = gemm<false, false>(b.dO, kOutPad, W[3], kHidden, rows, kHidden, kOutPad, d, s);
    if (rc) return rc;
  }
  for (int l = 2; l >= 0; --l) {
    gelu_back_kernel<<<grid1(rows * kHidden), 256, 0, s>>>(b.dA, b.Z[l], rows * kHidden, b.dZ);
    ++g_launches;
    const bf16* prev = l > 0 ? b.A[l - 1] : X;
    const int kin = l > 0 ? kHidden : kIn;
    Epi e{grad + param_offset(l, false), kin, nullptr, 0, nullptr, 0, nullptr, 0, 1, err};
    rc = gemm<true, false>(b.dZ, kHidden, prev, kin, kHidden, kin, rows, e, s, kchunk);
    if (rc) return rc;
    bias_grad_kernel<<<kHidden, 256, 0, s>>>(b.dZ, rows, kHidden, grad + param_offset(l, true));
    ++g_launches;
    if (l > 0) {
      Epi d{b.dA, kHidden, nullptr, 0, nullptr, 0, nullptr, 0, 0, err};
      rc = gemm<false, false>(b.dZ, kHidden, W[l], kin, rows, kin, kHidden, d, s);
      if (rc) return rc;
    }
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(QBC_E_CUDA, "mlp gradient: %s", cudaGetErrorString(e));
  return QBC_OK;
}

int Net::adam(float lr, cudaStream_t s) {
  ++step_count;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.0f - std::pow(b1, (float)step_count), c2 = 1.0f - std::pow(b2, (float)step_count);
  const int64_t n = param_count();
  adam_kernel<<<grid1(n), 256, 0, s>>>(master, grad, m, v, n, lr, b1, b2, 1e-8f, c1, c2);
  ++g_launches;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(QBC_E_CUDA, "mlp adam: %s", cudaGetErrorString(e));
  return sync_weights(s);
}

}  // namespace mlp
}  // namespace qbc
