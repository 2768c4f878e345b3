// Occluder-proposal network (mlp.cu): sizes, parameter layout and the
// device-side state a context keeps.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace qbc {
namespace mlp {

constexpr int kInUsed = 45;   // 9 features + 6-frequency sin/cos of the hit point
constexpr int kIn = 48;       // padded to a multiple of 16
constexpr int kHidden = 128;
constexpr int kOut = 3;       // proposed t along the shadow ray
constexpr int kGate = 3;      // output 3: logit of "the shadow ray is occluded before the hit"
constexpr int kOutUsed = 4;
constexpr int kOutPad = 16;
constexpr float kGateWeight = 0.05f;  // weight of the gate's cross-entropy in the loss
constexpr int64_t kChunkRows = 1 << 20;  // inference rows per pass through the work buffer

int64_t param_offset(int layer, bool bias);  // floats into the master array
int64_t param_count();
int64_t launches();  // kernels this thread has launched through the network so far

struct Net {
  float* master = nullptr;       // fp32 parameters (W1 b1 W2 b2 W3 b3 W4 b4, W as [out][in])
  __nv_bfloat16* wb = nullptr;   // bf16 copy used by the kernels (same layout)
  float* grad = nullptr;
  float* m = nullptr;            // Adam moments
  float* v = nullptr;
  void* work = nullptr;          // activations of a batch
  int64_t work_rows = 0;
  int64_t step_count = 0;
  bool ready = false;
  unsigned* err = nullptr;       // device error word of the owning context

  int init(uint64_t seed, cudaStream_t s);
  int set(const float* host, cudaStream_t s);
  int get(float* host, cudaStream_t s) const;
  int sync_weights(cudaStream_t s);
  int ensure_work(int64_t rows);
  // out: rows x kOutPad fp32; keep: retain activations for gradient()
  int forward(const __nv_bfloat16* X, int64_t rows, float* out, cudaStream_t s, bool keep = false);
  // loss (device float, mean over rows) and parameter gradient into grad
  int gradient(const __nv_bfloat16* X, const float* tlab, const int8_t* kind, int64_t rows, float* loss,
               cudaStream_t s);
  int adam(float lr, cudaStream_t s);
  void release();
};

}  // namespace mlp
}  // namespace qbc
