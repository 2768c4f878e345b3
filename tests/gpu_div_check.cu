// Checks div_by_recip (qubatron_gb300/csrc/trace.cuh) against IEEE division
// (a / b with -prec-div=true) bit for bit over the operand ranges its callers
// allow (recip_div_ok): |b| in [2^-40, 2^40], |a| zero or in [2^-62, 2^65],
// plus numerators of the traversal's form (a cube midpoint minus a ray
// origin). Prints "checked N mismatches M first a b got want".
#include <cstdio>
#include <cstdint>

#include "trace.cuh"

__device__ __forceinline__ uint64_t mix(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__device__ float rand_float(uint64_t r, int emin, int emax) {
  const uint32_t m = (uint32_t)(r & 0x7FFFFFu);
  const int e = emin + (int)((r >> 23) % (uint64_t)(emax - emin + 1));
  const uint32_t s = (uint32_t)((r >> 40) & 1u) << 31;
  return __uint_as_float(s | ((uint32_t)(e + 127) << 23) | m);
}

__global__ void check(uint64_t n, uint64_t seed, unsigned long long* bad, float* first) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t r1 = mix(seed + 0x9E3779B97F4A7C15ull * (2 * i + 1)), r2 = mix(r1 ^ 0x5851F42D4C957F2Dull);
    const float b = rand_float(r2, -40, 39);
    float a;
    if ((i & 3) == 0) {
      // a cube midpoint (2k+1) S / 2^(L+1), S = 1800, minus an origin
      const int L = (int)(r1 % 18u);
      const uint32_t k = (uint32_t)((r1 >> 8) % (1u << L));
      const float c = (float)(2 * k + 1) * (1800.0f / (float)(2u << L));
      const float p = rand_float(r1 >> 20, -30, 12);
      a = c - p;
    } else if ((i & 255) == 1) {
      a = 0.0f;
    } else {
      a = rand_float(r1, -62, 64);
    }
    const float want = a / b;
    const float got = qbc::div_by_recip(a, b, 1.0f / b);
    if (__float_as_uint(got) != __float_as_uint(want)) {
      if (atomicAdd(bad, 1ull) == 0) {
        first[0] = a;
        first[1] = b;
        first[2] = got;
        first[3] = want;
      }
    }
  }
}

int main(int argc, char** argv) {
  const uint64_t n = argc > 1 ? strtoull(argv[1], nullptr, 10) : (1ull << 32);
  unsigned long long* bad;
  float* first;
  cudaMalloc(&bad, sizeof(unsigned long long));
  cudaMalloc(&first, 4 * sizeof(float));
  cudaMemset(bad, 0, sizeof(unsigned long long));
  check<<<152 * 16, 256>>>(n, 20261204ull, bad, first);
  unsigned long long h = 0;
  float f[4] = {0, 0, 0, 0};
  cudaMemcpy(&h, bad, sizeof(h), cudaMemcpyDeviceToHost);
  cudaMemcpy(f, first, sizeof(f), cudaMemcpyDeviceToHost);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    printf("cuda error %s\n", cudaGetErrorString(e));
    return 2;
  }
  printf("checked %llu mismatches %llu first %.9g %.9g %.9g %.9g\n", (unsigned long long)n, h, f[0], f[1], f[2],
         f[3]);
  return h == 0 ? 0 : 1;
}
