// The occluder-proposal network inside libqbcuda: features of shade-pass
// records, the training set logged by plain renders, the fused inference
// kernel launch behind QBC_PROPOSE_MLP, and the qbc_proposal_* entry points.
// The network's own kernels are in mlp.cu and mlp_device.cuh.

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <new>
#include <vector>

#include "mlp_device.cuh"
#include "qbc_ctx.h"

// ---------------------------------------------------------------------------
// Occluder-proposal network: features, dataset, training, inference
// ---------------------------------------------------------------------------

namespace {

using bf16 = __nv_bfloat16;

// Network input of a shade-pass record: hit point normalised to the
// basecube, unit normal, unit direction to the light, and sin/cos of pi
// times the normalised hit point scaled by 4, 8, ..., 128 (45 values, zero
// padded). The normal is the primary leaf's, fetched again as the render
// fetched it.
__device__ __forceinline__ void record_features(const qbc::DevScene& sc, const qbc::Batch& b, const uint32_t* r,
                                                bf16* x) {
  const qbc_view& v = b.job[r[qbc::kRecView] & 0xFFu].v;
  const float S = v.basecube[3];
  const float lo[3] = {v.basecube[0], v.basecube[1] - S, v.basecube[2] - S};
  float4 col = make_float4(0.0f, 0.0f, 0.0f, 0.0f), nrm = col;
  if (r[qbc::kRecFlags] & QBC_PX_PRIMARY_LEAF)
    qbc::leaf_texel(sc, sc.tree[1].n > 0, (int32_t)r[qbc::kRecLeaf], (int32_t)r[qbc::kRecLeaf + 1], v.maxlevel, col,
                    nrm);
  float f[qbc::mlp::kIn];
  float isp[3], n[3] = {nrm.x, nrm.y, nrm.z}, l[3];
  for (int k = 0; k < 3; ++k) {
    isp[k] = __uint_as_float(r[qbc::kRecIsp + k]);
    l[k] = v.light[k] - isp[k];
  }
  const float nn = rsqrtf(fmaxf(n[0] * n[0] + n[1] * n[1] + n[2] * n[2], 1e-20f));
  const float ll = rsqrtf(fmaxf(l[0] * l[0] + l[1] * l[1] + l[2] * l[2], 1e-20f));
  for (int k = 0; k < 3; ++k) {
    f[k] = (isp[k] - lo[k]) / S;
    f[3 + k] = n[k] * nn;
    f[6 + k] = l[k] * ll;
  }
  int o = 9;
  for (int q = 0; q < 6; ++q) {
    const float sc = (float)(4 << q);
    for (int k = 0; k < 3; ++k) {
      f[o++] = sinpif(sc * f[k]);
      f[o++] = cospif(sc * f[k]);
    }
  }
  for (; o < qbc::mlp::kIn; ++o) f[o] = 0.0f;
  for (int k = 0; k < qbc::mlp::kIn; ++k) x[k] = __float2bfloat16(f[k]);
}

// Shaded records of a logged render -> training samples (appended).
__global__ void collect_kernel(const qbc::DevScene sc, const __grid_constant__ qbc::Batch b,
                               const __grid_constant__ qbc::Wave w,
                               bf16* __restrict__ X, float* __restrict__ tl, int8_t* __restrict__ kind,
                               unsigned int* __restrict__ count, int64_t cap) {
  const unsigned total = min(*w.qcount, w.cap);
  for (unsigned q = blockIdx.x * blockDim.x + threadIdx.x; q < total; q += gridDim.x * blockDim.x) {
    const uint32_t* r = w.rec + (size_t)q * qbc::kRecWords;
    if (!(r[qbc::kRecFlags] & QBC_PX_SHADED)) continue;
    const float t = __uint_as_float(r[qbc::kRecLogT]);
    const bool lit = r[qbc::kRecLogLit] != 0;
    const bool occluded = !lit && t > 0.0f && t < 1.0f;
    if (!lit && !occluded) continue;  // unlit without an occluder before the hit: no label
    const unsigned i = atomicAdd(count, 1u);
    if ((int64_t)i >= cap) continue;
    record_features(sc, b, r, X + (size_t)i * qbc::mlp::kIn);
    tl[i] = occluded ? t : 2.0f;
    kind[i] = occluded ? 1 : 0;
  }
}

// Fused-network rows over the shade-pass record queue: the features of each
// record in, its proposals out (earliest first; none where the occlusion
// logit is below the gate). The row count is read on the device.
struct RecordRows {
  qbc::DevScene sc;
  qbc::Batch b;
  qbc::Wave w;
  float gate;
  int keep;  // proposals kept, earliest first
  __device__ __forceinline__ uint32_t rows() const { return min(*w.qcount, w.cap); }
  __device__ __forceinline__ void load(uint32_t r0, uint32_t n, bf16* x, int lane) const {
    if (lane >= 16) return;
    bf16* row = x + lane * qbc::mlp::kLdIn;
    if ((uint32_t)lane < n) {
      record_features(sc, b, w.rec + (size_t)(r0 + lane) * qbc::kRecWords, row);
    } else {
      for (int k = 0; k < qbc::mlp::kIn; ++k) row[k] = __float2bfloat16(0.0f);
    }
  }
  __device__ __forceinline__ void store(uint32_t r, const float* o) const {
    float t[3] = {o[0], o[1], o[2]};
    if (!(o[qbc::mlp::kGate] >= gate)) t[0] = t[1] = t[2] = -1.0f;
    for (int i = 0; i < 2; ++i)
      for (int j = i + 1; j < 3; ++j)
        if (t[j] < t[i]) {
          const float x = t[i];
          t[i] = t[j];
          t[j] = x;
        }
    for (int k = keep; k < 3; ++k) t[k] = -1.0f;
    uint32_t* rec = w.rec + (size_t)r * qbc::kRecWords;
    for (int k = 0; k < 3; ++k) rec[qbc::kRecProp + k] = __float_as_uint(t[k]);
  }
};

// Fused-network rows over a bf16 feature matrix (kIn per row) -> kOutUsed
// floats per row.
struct MatrixRows {
  const bf16* X;
  float* out;
  uint32_t m;
  __device__ __forceinline__ uint32_t rows() const { return m; }
  __device__ __forceinline__ void load(uint32_t r0, uint32_t n, bf16* x, int lane) const {
    constexpr int kVec = qbc::mlp::kIn / 8;
    for (int e = lane; e < 16 * kVec; e += 32) {
      const int r = e / kVec, c = e % kVec;
      uint4 v = make_uint4(0u, 0u, 0u, 0u);
      if ((uint32_t)r < n) v = reinterpret_cast<const uint4*>(X + (size_t)(r0 + r) * qbc::mlp::kIn)[c];
      *reinterpret_cast<uint4*>(x + r * qbc::mlp::kLdIn + c * 8) = v;
    }
  }
  __device__ __forceinline__ void store(uint32_t r, const float* o) const {
    for (int k = 0; k < qbc::mlp::kOutUsed; ++k) out[(size_t)r * qbc::mlp::kOutUsed + k] = o[k];
  }
};

// Random minibatch of the training set.
__global__ void gather_kernel(const bf16* __restrict__ X, const float* __restrict__ tl,
                              const int8_t* __restrict__ kind, int64_t n, int64_t rows, uint64_t seed,
                              bf16* __restrict__ bx, float* __restrict__ bt, int8_t* __restrict__ bk) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < rows; i += (int64_t)gridDim.x * blockDim.x) {
    uint64_t z = seed + 0x9E3779B97F4A7C15ull * (uint64_t)(i + 1);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    const int64_t j = (int64_t)(z % (uint64_t)n);
    for (int k = 0; k < qbc::mlp::kIn; ++k) bx[i * qbc::mlp::kIn + k] = X[j * qbc::mlp::kIn + k];
    bt[i] = tl[j];
    bk[i] = kind[j];
  }
}

bf16 host_bf16(float f) {
  // round to nearest even (NaN kept quiet)
  uint32_t u;
  std::memcpy(&u, &f, 4);
  if ((u & 0x7fffffffu) > 0x7f800000u) return __ushort_as_bfloat16((unsigned short)((u >> 16) | 0x40));
  u += 0x7fffu + ((u >> 16) & 1u);
  return __ushort_as_bfloat16((unsigned short)(u >> 16));
}

// One launch of the network over `src`'s rows on the tcgen05 tensor cores: a
// persistent grid of one block per SM, each staging the weights once.
template <class Src>
int launch_fused(qbc_ctx* c, const Src& src, int variant) {
  auto kern = qbc::mlp::umma_forward_kernel<Src>;
  const int smem = (int)qbc::mlp::kUmmaSmemBytes;
  if (!c->fused_attr[variant]) {
    QBC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    c->fused_attr[variant] = true;
  }
  int per_sm = 0;
  QBC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, qbc::mlp::kUmmaThreads, smem));
  if (per_sm < 1) return fail(QBC_E_STATE, "proposal network: no block fits on an SM");
  qbc::mlp::FusedParams p;
  for (int l = 0; l < 4; ++l) {
    p.w[l] = c->net.wb + qbc::mlp::param_offset(l, false);
    p.b[l] = c->net.master + qbc::mlp::param_offset(l, true);
    if (reinterpret_cast<uintptr_t>(p.w[l]) % 16) return fail(QBC_E_STATE, "proposal network: unaligned weights");
  }
  // one block per SM: each holds 256 of the SM's 512 tensor-memory columns
  kern<<<c->sm_count, qbc::mlp::kUmmaThreads, smem, c->stream>>>(p, src, c->derr);
  QBC_CUDA(cudaGetLastError());
  ++c->launches;
  return QBC_OK;
}


int ensure_dataset(qbc_ctx* c, int64_t cap) {
  if (c->ds_cap >= cap) return QBC_OK;
  // grow keeping the samples collected so far
  bf16* x = nullptr;
  float* t = nullptr;
  int8_t* k = nullptr;
  cudaError_t e = cudaMalloc(&x, (size_t)cap * qbc::mlp::kIn * 2);
  if (e == cudaSuccess) e = cudaMalloc(&t, (size_t)cap * 4);
  if (e == cudaSuccess) e = cudaMalloc(&k, (size_t)cap);
  if (e == cudaSuccess && !c->ds_count) e = cudaMalloc(&c->ds_count, sizeof(unsigned));
  if (e != cudaSuccess) {
    cudaFree(x);
    cudaFree(t);
    cudaFree(k);
    return fail(QBC_E_NOMEM, "proposal training set of %lld samples: %s", (long long)cap, cudaGetErrorString(e));
  }
  unsigned have = 0;
  if (c->ds_cap > 0) {
    QBC_CUDA(cudaMemcpyAsync(&have, c->ds_count, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
    QBC_CUDA(cudaStreamSynchronize(c->stream));
    have = (unsigned)std::min<int64_t>(have, c->ds_cap);
    QBC_CUDA(cudaMemcpyAsync(x, c->ds_x, (size_t)have * qbc::mlp::kIn * 2, cudaMemcpyDeviceToDevice, c->stream));
    QBC_CUDA(cudaMemcpyAsync(t, c->ds_t, (size_t)have * 4, cudaMemcpyDeviceToDevice, c->stream));
    QBC_CUDA(cudaMemcpyAsync(k, c->ds_kind, (size_t)have, cudaMemcpyDeviceToDevice, c->stream));
    QBC_CUDA(cudaStreamSynchronize(c->stream));
  }
  cudaFree(c->ds_x);
  cudaFree(c->ds_t);
  cudaFree(c->ds_kind);
  c->ds_x = x;
  c->ds_t = t;
  c->ds_kind = k;
  c->ds_cap = cap;
  QBC_CUDA(cudaMemcpyAsync(c->ds_count, &have, sizeof(unsigned), cudaMemcpyHostToDevice, c->stream));
  QBC_CUDA(cudaStreamSynchronize(c->stream));
  return QBC_OK;
}

}  // namespace

// Proposals of every queued record from the network (no host round trip:
// the kernel reads the queue length on the device).
int propose_mlp(qbc_ctx* c, const qbc::Batch& b, const qbc::Wave& w) {
  if (!c->net.ready) return fail(QBC_E_STATE, "qbc_render_views_ex: no occluder network in this context");
  std::unique_ptr<RecordRows> src(new RecordRows());
  src->sc = device_scene(c);
  src->b = b;
  src->w = w;
  const float p = (float)c->proposal_gate * 1e-3f;  // gate probability -> logit
  src->gate = c->proposal_gate <= 0 ? -INFINITY : logf(p / (1.0f - p));
  src->keep = c->proposal_count;
  return launch_fused(c, *src, 0);
}

// ---------------------------------------------------------------------------
// Occluder-proposal network: C ABI
// ---------------------------------------------------------------------------

namespace {
// Host rows of 45 floats -> device bf16 rows of 48.
int upload_features(qbc_ctx* c, const float* x, int64_t m, bf16** out) {
  std::vector<bf16> h((size_t)m * qbc::mlp::kIn);
  for (int64_t i = 0; i < m; ++i)
    for (int k = 0; k < qbc::mlp::kIn; ++k)
      h[(size_t)i * qbc::mlp::kIn + k] = host_bf16(k < qbc::mlp::kInUsed ? x[i * qbc::mlp::kInUsed + k] : 0.0f);
  cudaError_t e = cudaMalloc(out, h.size() * 2);
  if (e != cudaSuccess) return fail(QBC_E_NOMEM, "proposal features: %s", cudaGetErrorString(e));
  QBC_CUDA(cudaMemcpyAsync(*out, h.data(), h.size() * 2, cudaMemcpyHostToDevice, c->stream));
  return QBC_OK;
}
}  // namespace

static_assert(QBC_PROPOSAL_PARAMS == 41360, "parameter count");

extern "C" int qbc_proposal_collect(qbc_ctx* c, const qbc_view* views, int n, int64_t* samples) {
  qbc::clear_error();
  if (!c || n < 0 || (n > 0 && !views)) return fail(QBC_E_ARG, "qbc_proposal_collect: bad argument");
  if (n > qbc::kMaxViewsPerLaunch)
    return fail(QBC_E_ARG, "qbc_proposal_collect: at most %d views per call", qbc::kMaxViewsPerLaunch);
  QBC_CUDA(cudaSetDevice(c->device));
  int64_t pixels = 0;
  for (int i = 0; i < n; ++i) {
    int rc = check_view(views[i], i);
    if (rc) return rc;
    pixels += (int64_t)views[i].width_px * views[i].height_px;
  }
  int rc = ensure_dataset(c, std::max<int64_t>(c->ds_cap, c->ds_cap == 0 ? pixels : 0));
  if (rc) return rc;
  if (n > 0) {
    std::vector<qbc_outputs> none(n);
    std::memset(none.data(), 0, sizeof(qbc_outputs) * n);
    qbc_render_opts o;
    std::memset(&o, 0, sizeof(o));
    o.two_pass = 1;
    o.log = 1;
    rc = render_views_impl(c, views, none.data(), n, 1, &o, nullptr);
    if (rc) return rc;
    // room for every shaded pixel of this batch
    unsigned have = 0, queued = 0;
    QBC_CUDA(cudaMemcpyAsync(&have, c->ds_count, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
    QBC_CUDA(cudaMemcpyAsync(&queued, c->wcount, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
    QBC_CUDA(cudaStreamSynchronize(c->stream));
    rc = ensure_dataset(c, std::max<int64_t>(c->ds_cap, (int64_t)have + queued));
    if (rc) return rc;
    // rebuild the batch parameters of that render for the feature kernel
    qbc::Batch* b = new qbc::Batch();
    for (int i = 0; i < n; ++i) b->job[i].v = views[i];
    b->n = n;
    qbc::Wave w{};
    w.rec = c->rec;
    w.qcount = c->wcount;
    w.cap = (uint32_t)std::min<int64_t>(c->rec_cap, 0xFFFFFFFFll);
    collect_kernel<<<launch_grid(c, queued), 256, 0, c->stream>>>(device_scene(c), *b, w, c->ds_x, c->ds_t,
                                                                  c->ds_kind, c->ds_count, c->ds_cap);
    delete b;
    QBC_CUDA(cudaGetLastError());
    ++c->launches;
  }
  unsigned cnt = 0;
  if (c->ds_count) {
    QBC_CUDA(cudaMemcpyAsync(&cnt, c->ds_count, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
    QBC_CUDA(cudaStreamSynchronize(c->stream));
  }
  if (samples) *samples = std::min<int64_t>(cnt, c->ds_cap);
  return QBC_OK;
}

extern "C" int qbc_proposal_train(qbc_ctx* c, const qbc_train_opts* opts, qbc_train_stats* stats) {
  qbc::clear_error();
  if (!c || !opts) return fail(QBC_E_ARG, "qbc_proposal_train: null argument");
  if (opts->steps < 0 || opts->batch < 64 || opts->batch > (1 << 22) || !(opts->lr > 0.0f))
    return fail(QBC_E_ARG, "qbc_proposal_train: steps >= 0, batch 64..4M and lr > 0 required");
  QBC_CUDA(cudaSetDevice(c->device));
  unsigned cnt = 0;
  if (c->ds_count) {
    QBC_CUDA(cudaMemcpyAsync(&cnt, c->ds_count, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
    QBC_CUDA(cudaStreamSynchronize(c->stream));
  }
  const int64_t n = std::min<int64_t>(cnt, c->ds_cap);
  if (n == 0) return fail(QBC_E_STATE, "qbc_proposal_train: empty training set (qbc_proposal_collect first)");
  if (!c->net.ready) {
    int rc = c->net.init(opts->seed, c->stream);
    if (rc) return rc;
  }
  const int64_t B = opts->batch;
  bf16* bx = nullptr;
  float* bt = nullptr;
  int8_t* bk = nullptr;
  float* dloss = nullptr;
  cudaError_t e = cudaMalloc(&bx, (size_t)B * qbc::mlp::kIn * 2);
  if (e == cudaSuccess) e = cudaMalloc(&bt, (size_t)B * 4);
  if (e == cudaSuccess) e = cudaMalloc(&bk, (size_t)B);
  if (e == cudaSuccess) e = cudaMalloc(&dloss, 4);
  int rc = QBC_OK;
  if (e != cudaSuccess) rc = fail(QBC_E_NOMEM, "qbc_proposal_train: %s", cudaGetErrorString(e));
  float first = 0.0f, last = 0.0f;
  int nlast = 0;
  for (int step = 0; step < opts->steps && rc == QBC_OK; ++step) {
    gather_kernel<<<launch_grid(c, B), 256, 0, c->stream>>>(c->ds_x, c->ds_t, c->ds_kind, n, B,
                                                            opts->seed * 1000003ull + (uint64_t)step, bx, bt, bk);
    const int64_t l0 = qbc::mlp::launches();
    rc = c->net.gradient(bx, bt, bk, B, dloss, c->stream);
    if (rc) break;
    rc = c->net.adam(opts->lr, c->stream);
    if (rc) break;
    c->launches += 1 + (qbc::mlp::launches() - l0);
    if (step == 0 || step >= opts->steps - 10) {
      float l = 0.0f;
      e = cudaMemcpyAsync(&l, dloss, 4, cudaMemcpyDeviceToHost, c->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
      if (e != cudaSuccess) {
        rc = fail(QBC_E_CUDA, "qbc_proposal_train: %s", cudaGetErrorString(e));
        break;
      }
      if (step == 0) first = l;
      if (step >= opts->steps - 10) {
        last += l;
        ++nlast;
      }
    }
  }
  cudaStreamSynchronize(c->stream);
  cudaFree(bx);
  cudaFree(bt);
  cudaFree(bk);
  cudaFree(dloss);
  if (rc) return rc;
  if (stats) {
    std::vector<int8_t> k((size_t)n);
    QBC_CUDA(cudaMemcpy(k.data(), c->ds_kind, (size_t)n, cudaMemcpyDeviceToHost));
    uint64_t occ = 0;
    for (int8_t v : k) occ += v == 1;
    stats->samples = (uint64_t)n;
    stats->occluded = occ;
    stats->loss_first = first;
    stats->loss_last = nlast ? last / nlast : first;
  }
  return QBC_OK;
}

extern "C" int qbc_proposal_clear(qbc_ctx* c) {
  if (!c) return fail(QBC_E_ARG, "qbc_proposal_clear: null context");
  if (c->ds_count) {
    QBC_CUDA(cudaMemsetAsync(c->ds_count, 0, sizeof(unsigned), c->stream));
    QBC_CUDA(cudaStreamSynchronize(c->stream));
  }
  return QBC_OK;
}

extern "C" int qbc_proposal_get_params(qbc_ctx* c, float* params) {
  qbc::clear_error();
  if (!c || !params) return fail(QBC_E_ARG, "qbc_proposal_get_params: null argument");
  if (!c->net.ready) return fail(QBC_E_STATE, "qbc_proposal_get_params: no network");
  QBC_CUDA(cudaSetDevice(c->device));
  return c->net.get(params, c->stream);
}

extern "C" int qbc_proposal_set_params(qbc_ctx* c, const float* params) {
  qbc::clear_error();
  if (!c || !params) return fail(QBC_E_ARG, "qbc_proposal_set_params: null argument");
  QBC_CUDA(cudaSetDevice(c->device));
  int rc = c->net.set(params, c->stream);
  if (rc) return rc;
  QBC_CUDA(cudaStreamSynchronize(c->stream));
  return QBC_OK;
}

extern "C" int qbc_proposal_eval(qbc_ctx* c, const float* x, int64_t m, float* out) {
  qbc::clear_error();
  if (!c || (m > 0 && (!x || !out)) || m < 0 || m > (1ll << 31))
    return fail(QBC_E_ARG, "qbc_proposal_eval: bad argument");
  if (!c->net.ready) return fail(QBC_E_STATE, "qbc_proposal_eval: no network");
  if (m == 0) return QBC_OK;
  QBC_CUDA(cudaSetDevice(c->device));
  bf16* dx = nullptr;
  int rc = upload_features(c, x, m, &dx);
  if (rc) return rc;
  float* dout = nullptr;
  cudaError_t e = cudaMalloc(&dout, (size_t)m * qbc::mlp::kOutUsed * 4);
  if (e != cudaSuccess) {
    cudaFree(dx);
    return fail(QBC_E_NOMEM, "qbc_proposal_eval: %s", cudaGetErrorString(e));
  }
  MatrixRows src{dx, dout, (uint32_t)m};
  rc = launch_fused(c, src, 1);
  if (!rc) {
    e = cudaMemcpyAsync(out, dout, (size_t)m * qbc::mlp::kOutUsed * 4, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) rc = fail(QBC_E_CUDA, "qbc_proposal_eval: %s", cudaGetErrorString(e));
  }
  cudaFree(dx);
  cudaFree(dout);
  return rc;
}

extern "C" int qbc_proposal_gradient(qbc_ctx* c, const float* x, const float* t, const int8_t* kind, int64_t m,
                                     float* loss, float* grad) {
  qbc::clear_error();
  if (!c || m <= 0 || !x || !t || !kind || !loss || !grad) return fail(QBC_E_ARG, "qbc_proposal_gradient: bad argument");
  if (!c->net.ready) return fail(QBC_E_STATE, "qbc_proposal_gradient: no network");
  QBC_CUDA(cudaSetDevice(c->device));
  bf16* dx = nullptr;
  int rc = upload_features(c, x, m, &dx);
  if (rc) return rc;
  float* dt = nullptr;
  int8_t* dk = nullptr;
  float* dl = nullptr;
  cudaError_t e = cudaMalloc(&dt, (size_t)m * 4);
  if (e == cudaSuccess) e = cudaMalloc(&dk, (size_t)m);
  if (e == cudaSuccess) e = cudaMalloc(&dl, 4);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dt, t, (size_t)m * 4, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dk, kind, (size_t)m, cudaMemcpyHostToDevice, c->stream);
  if (e != cudaSuccess) rc = fail(QBC_E_CUDA, "qbc_proposal_gradient: %s", cudaGetErrorString(e));
  if (!rc) rc = c->net.gradient(dx, dt, dk, m, dl, c->stream);
  if (!rc) {
    e = cudaMemcpyAsync(loss, dl, 4, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(grad, c->net.grad, (size_t)QBC_PROPOSAL_PARAMS * 4, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) rc = fail(QBC_E_CUDA, "qbc_proposal_gradient: %s", cudaGetErrorString(e));
  }
  cudaFree(dx);
  cudaFree(dt);
  cudaFree(dk);
  cudaFree(dl);
  return rc;
}
