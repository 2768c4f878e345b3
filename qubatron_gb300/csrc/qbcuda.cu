// libqbcuda: context, uploads and the render kernel behind include/qbcuda.h.
//
// The kernels are in render.cuh (per-pixel shader body, persistent) and
// walker.cuh (the traversal). Build flags: -fmad=false -prec-div=true
// -prec-sqrt=true -ftz=false.

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <memory>
#include <new>
#include <vector>

#include "qbc_internal.h"
#include "qbcuda.h"
#include "mlp.h"
#include "mlp_device.cuh"
#include "render.cuh"

using qbc::fail;

namespace qbc {

// Split 12-int nodes (octree.c:11-14) into 32-byte child blocks + model index.
__global__ void repack_nodes_kernel(const int4* __restrict__ raw, int64_t n, int4* __restrict__ child,
                                    int32_t* __restrict__ model) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    int4 a = raw[3 * i], b = raw[3 * i + 1], c = raw[3 * i + 2];
    child[2 * i] = a;
    child[2 * i + 1] = b;
    model[i] = c.x;
  }
}

// float3 points -> float4 texels; w = 1 as an RGB32F texel reads (colour and normal alike).
__global__ void expand_attr_kernel(const float* __restrict__ raw, int64_t n, float4* __restrict__ out, float w) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = make_float4(raw[3 * i], raw[3 * i + 1], raw[3 * i + 2], w);
}

}  // namespace qbc

// ---------------------------------------------------------------------------
// Context
// ---------------------------------------------------------------------------

struct DevTreeBuf {
  int4* child = nullptr;
  int32_t* model = nullptr;
  int64_t n = 0;    // node count of the array last uploaded
  int64_t cap = 0;  // nodes allocated
};

struct DevModelBuf {
  float4* col = nullptr;
  float4* nrm = nullptr;
  int64_t n_col = 0, n_nrm = 0;
  int64_t cap_col = 0, cap_nrm = 0;
};

struct qbc_ctx {
  int device = 0;
  int sm_count = 0;
  cudaStream_t own = nullptr;
  cudaStream_t stream = nullptr;
  DevTreeBuf tree[2];
  DevModelBuf model[2];
  void* stage = nullptr;  // device staging for uploads
  size_t stage_bytes = 0;
  void* scratch = nullptr;  // device outputs for host-output renders
  size_t scratch_bytes = 0;
  unsigned int* queue = nullptr;  // global tile counter of the persistent render kernel
  // two-pass render: records, counters (queued, shade-pass next), statistics, per-pixel log
  uint32_t* rec = nullptr;
  int64_t rec_cap = 0;
  unsigned int* wcount = nullptr;
  unsigned long long* wstats = nullptr;
  float* pixlog = nullptr;
  int64_t pixlog_cap = 0;
  int64_t pixlog_valid = 0;  // pixels of the last logged render (0: none)
  // occluder-proposal network and its training set
  qbc::mlp::Net net;
  __nv_bfloat16* ds_x = nullptr;  // features, kIn per sample
  float* ds_t = nullptr;          // first-occluder t
  int8_t* ds_kind = nullptr;      // 1 occluded, 0 lit
  int64_t ds_cap = 0;
  unsigned int* ds_count = nullptr;
  bool fused_attr[2] = {false, false};  // dynamic shared memory set for the fused network kernels
  std::vector<qbc_graph*> graphs;       // captured frames, detached when the context goes
  int render_blocks[4] = {0, 0, 0, 0};  // resident blocks per SM of each render_kernel variant
  int attr_done = 0;
  int service_min = qbc::kServiceMinDefault;
  int tile_shift = 3;     // 8x4 warp tiles
  int blocks_per_sm = 0;  // render blocks per SM (0: as many as fit)
  int proposal_gate = 500;  // per mille: minimum predicted occlusion probability to try a proposal
  int proposal_count = 3;   // network proposals tried per pixel (earliest first)
  int64_t launches = 0;
};

namespace {

constexpr size_t kStageMax = size_t(256) << 20;

int cuda_fail(cudaError_t e, const char* what) {
  return fail(QBC_E_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define QBC_CUDA(call)                            \
  do {                                            \
    cudaError_t e_ = (call);                      \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
  } while (0)

int ensure_stage(qbc_ctx* c, size_t bytes) {
  if (c->stage_bytes >= bytes) return QBC_OK;
  if (c->stage) QBC_CUDA(cudaFree(c->stage));
  c->stage = nullptr;
  c->stage_bytes = 0;
  cudaError_t e = cudaMalloc(&c->stage, bytes);
  if (e != cudaSuccess) return fail(QBC_E_NOMEM, "staging buffer of %zu bytes: %s", bytes, cudaGetErrorString(e));
  c->stage_bytes = bytes;
  return QBC_OK;
}

template <typename T>
int grow(T** p, int64_t* cap, int64_t need, size_t elem_bytes, const char* what) {
  if (*cap >= need) return QBC_OK;
  if (*p) QBC_CUDA(cudaFree(*p));
  *p = nullptr;
  *cap = 0;
  cudaError_t e = cudaMalloc((void**)p, (size_t)need * elem_bytes);
  if (e != cudaSuccess)
    return fail(QBC_E_NOMEM, "%s: %lld items: %s", what, (long long)need, cudaGetErrorString(e));
  *cap = need;
  return QBC_OK;
}

int launch_grid(const qbc_ctx* c, int64_t n) {
  int64_t blocks = (n + 255) / 256;
  int64_t maxb = (int64_t)std::max(c->sm_count, 1) * 16;
  return (int)std::max<int64_t>(1, std::min(blocks, maxb));
}

qbc::DevScene device_scene(const qbc_ctx* c) {
  qbc::DevScene s;
  for (int t = 0; t < 2; ++t) {
    s.tree[t].child = c->tree[t].child;
    s.tree[t].model = c->tree[t].model;
    s.tree[t].n = (int32_t)c->tree[t].n;
    s.model[t].col = c->model[t].col;
    s.model[t].nrm = c->model[t].nrm;
    // the colour and normal arrays are separate uploads; a point index is
    // valid when both hold it
    s.model[t].n = (int32_t)std::min(c->model[t].n_col, c->model[t].n_nrm);
  }
  return s;
}

}  // namespace

extern "C" int qbc_create(int device, qbc_ctx** out) {
  qbc::clear_error();
  if (!out) return fail(QBC_E_ARG, "qbc_create: null out");
  *out = nullptr;
  int ndev = 0;
  QBC_CUDA(cudaGetDeviceCount(&ndev));
  if (device < 0 || device >= ndev) return fail(QBC_E_ARG, "qbc_create: device %d of %d", device, ndev);
  QBC_CUDA(cudaSetDevice(device));
  qbc_ctx* c = new qbc_ctx();
  c->device = device;
  cudaError_t e = cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete c;
    return cuda_fail(e, "qbc_create");
  }
  if (e == cudaSuccess) e = cudaMalloc(&c->queue, sizeof(unsigned int));
  if (e == cudaSuccess) e = cudaMalloc(&c->wcount, 2 * sizeof(unsigned int));
  if (e == cudaSuccess) e = cudaMalloc(&c->wstats, qbc::kStatCount * sizeof(unsigned long long));
  if (e != cudaSuccess) {
    if (c->own) cudaStreamDestroy(c->own);
    delete c;
    return cuda_fail(e, "qbc_create");
  }
  c->stream = c->own;
  *out = c;
  return QBC_OK;
}

void detach_graph(qbc_graph* g);

extern "C" int qbc_destroy(qbc_ctx* c) {
  if (!c) return QBC_OK;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  for (qbc_graph* g : c->graphs) detach_graph(g);
  for (int t = 0; t < 2; ++t) {
    cudaFree(c->tree[t].child);
    cudaFree(c->tree[t].model);
    cudaFree(c->model[t].col);
    cudaFree(c->model[t].nrm);
  }
  cudaFree(c->stage);
  cudaFree(c->scratch);
  cudaFree(c->queue);
  c->net.release();
  cudaFree(c->ds_x);
  cudaFree(c->ds_t);
  cudaFree(c->ds_kind);
  cudaFree(c->ds_count);
  cudaFree(c->rec);
  cudaFree(c->wcount);
  cudaFree(c->wstats);
  cudaFree(c->pixlog);
  if (c->own) cudaStreamDestroy(c->own);
  delete c;
  return QBC_OK;
}

extern "C" int qbc_set_stream(qbc_ctx* c, void* stream) {
  if (!c) return fail(QBC_E_ARG, "qbc_set_stream: null context");
  c->stream = stream ? (cudaStream_t)stream : c->own;
  return QBC_OK;
}

extern "C" int qbc_set_option(qbc_ctx* c, int option, int value) {
  if (!c) return fail(QBC_E_ARG, "qbc_set_option: null context");
  if (option == QBC_OPT_SERVICE_MIN) {
    if (value < 1 || value > 32) return fail(QBC_E_ARG, "qbc_set_option: service threshold %d outside 1..32", value);
    c->service_min = value;
    return QBC_OK;
  }
  if (option == QBC_OPT_PROPOSAL_GATE) {
    if (value < 0 || value > 999) return fail(QBC_E_ARG, "qbc_set_option: proposal gate %d outside 0..999", value);
    c->proposal_gate = value;
    return QBC_OK;
  }
  if (option == QBC_OPT_PROPOSAL_COUNT) {
    if (value < 1 || value > 3) return fail(QBC_E_ARG, "qbc_set_option: proposal count %d outside 1..3", value);
    c->proposal_count = value;
    return QBC_OK;
  }
  if (option == QBC_OPT_TILE_WIDTH) {
    if (value != 2 && value != 4 && value != 8 && value != 16 && value != 32)
      return fail(QBC_E_ARG, "qbc_set_option: tile width %d (2, 4, 8, 16 or 32)", value);
    c->tile_shift = value == 2 ? 1 : value == 4 ? 2 : value == 8 ? 3 : value == 16 ? 4 : 5;
    return QBC_OK;
  }
  if (option == QBC_OPT_BLOCKS_PER_SM) {
    if (value < 0 || value > 32) return fail(QBC_E_ARG, "qbc_set_option: blocks per SM %d outside 0..32", value);
    c->blocks_per_sm = value;
    return QBC_OK;
  }
  return fail(QBC_E_ARG, "qbc_set_option: unknown option %d", option);
}

extern "C" int qbc_get_option(qbc_ctx* c, int option, int* value) {
  if (!c || !value) return fail(QBC_E_ARG, "qbc_get_option: null argument");
  if (option == QBC_OPT_SERVICE_MIN) {
    *value = c->service_min;
    return QBC_OK;
  }
  if (option == QBC_OPT_PROPOSAL_GATE) {
    *value = c->proposal_gate;
    return QBC_OK;
  }
  if (option == QBC_OPT_PROPOSAL_COUNT) {
    *value = c->proposal_count;
    return QBC_OK;
  }
  if (option == QBC_OPT_TILE_WIDTH) {
    *value = 1 << c->tile_shift;
    return QBC_OK;
  }
  if (option == QBC_OPT_BLOCKS_PER_SM) {
    *value = c->blocks_per_sm;
    return QBC_OK;
  }
  return fail(QBC_E_ARG, "qbc_get_option: unknown option %d", option);
}

extern "C" int qbc_synchronize(qbc_ctx* c) {
  if (!c) return fail(QBC_E_ARG, "qbc_synchronize: null context");
  QBC_CUDA(cudaStreamSynchronize(c->stream));
  return QBC_OK;
}

extern "C" int qbc_tree_nodes(qbc_ctx* c, int tree, int64_t* n) {
  if (!c || !n || tree < 0 || tree > 1) return fail(QBC_E_ARG, "qbc_tree_nodes: bad argument");
  *n = c->tree[tree].n;
  return QBC_OK;
}

extern "C" int qbc_model_points(qbc_ctx* c, int model, int64_t* n) {
  if (!c || !n || model < 0 || model > 1) return fail(QBC_E_ARG, "qbc_model_points: bad argument");
  *n = std::min(c->model[model].n_col, c->model[model].n_nrm);
  return QBC_OK;
}

extern "C" int qbc_launch_count(qbc_ctx* c, int64_t* count) {
  if (!c || !count) return fail(QBC_E_ARG, "qbc_launch_count: bad argument");
  *count = c->launches;
  return QBC_OK;
}

// ---------------------------------------------------------------------------
// Upload (octree_glc_upload_texbuffer_data, octree_glc.c:361-498)
// ---------------------------------------------------------------------------

namespace {
int upload_impl(qbc_ctx* c, const void* data, int type, size_t size, size_t itemsize, size_t start, size_t end,
                int buftype, bool device_src);
}

extern "C" int qbc_upload(qbc_ctx* c, const void* data, int type, size_t size, size_t itemsize, size_t start,
                          size_t end, int buftype) {
  qbc::clear_error();
  return upload_impl(c, data, type, size, itemsize, start, end, buftype, false);
}

extern "C" int qbc_upload_device(qbc_ctx* c, const void* data, int type, size_t size, size_t itemsize, size_t start,
                                 size_t end, int buftype) {
  qbc::clear_error();
  return upload_impl(c, data, type, size, itemsize, start, end, buftype, true);
}

namespace {
int upload_impl(qbc_ctx* c, const void* data, int type, size_t size, size_t itemsize, size_t start, size_t end,
                int buftype, bool device_src) {
  if (!c) return fail(QBC_E_ARG, "qbc_upload: null context");
  if (buftype < QBC_STATIC_COLOR || buftype > QBC_DYNAMIC_OCTREE)
    return fail(QBC_E_ARG, "qbc_upload: unknown buffer %d", buftype);
  if (start > end || end > size) return fail(QBC_E_ARG, "qbc_upload: range [%zu, %zu) outside size %zu", start, end, size);
  if (size > 0 && !data) return fail(QBC_E_ARG, "qbc_upload: null data");
  QBC_CUDA(cudaSetDevice(c->device));
  const char* base = static_cast<const char*>(data);
  const bool octree = buftype == QBC_STATIC_OCTREE || buftype == QBC_DYNAMIC_OCTREE;

  if (octree) {
    if (type != QBC_GL_INT) return fail(QBC_E_ARG, "qbc_upload: octree buffers take GL_INT data");
    if (itemsize != 16 && itemsize != 48)
      return fail(QBC_E_ARG, "qbc_upload: octree itemsize %zu (16 = one texel, 48 = one node)", itemsize);
    const size_t node_bytes = 48;
    const int64_t n_total = (int64_t)(size / node_bytes);
    if (n_total > INT32_MAX) return fail(QBC_E_ARG, "qbc_upload: %lld nodes exceed int32 indices", (long long)n_total);
    DevTreeBuf& t = c->tree[buftype == QBC_STATIC_OCTREE ? 0 : 1];
    int64_t lo = (int64_t)(start / node_bytes);
    int64_t hi = (int64_t)((end + node_bytes - 1) / node_bytes);
    if (n_total > t.cap) {
      // the reference re-creates the texture and refills it from [0, size)
      int64_t cap = n_total + n_total / 8;
      int rc = grow(&t.child, &t.cap, cap, 32, "octree child blocks");
      if (rc) return rc;
      int64_t mcap = 0;
      rc = grow(&t.model, &mcap, cap, 4, "octree model indices");
      if (rc) return rc;
      lo = 0;
      hi = n_total;
    }
    hi = std::min(hi, n_total);
    t.n = n_total;
    const int64_t chunk = (int64_t)(kStageMax / node_bytes);
    if (hi > lo && !device_src) {
      int rc = ensure_stage(c, (size_t)std::min(hi - lo, chunk) * node_bytes);
      if (rc) return rc;
    }
    for (int64_t a = lo; a < hi; a += chunk) {
      int64_t b = std::min(hi, a + chunk);
      const void* src = base + a * node_bytes;
      if (!device_src) {
        QBC_CUDA(cudaMemcpyAsync(c->stage, src, (size_t)(b - a) * node_bytes, cudaMemcpyHostToDevice, c->stream));
        src = c->stage;
      }
      qbc::repack_nodes_kernel<<<launch_grid(c, b - a), 256, 0, c->stream>>>(
          (const int4*)src, b - a, t.child + 2 * a, t.model + a);
      QBC_CUDA(cudaGetLastError());
      ++c->launches;
    }
  } else {
    if (type != QBC_GL_FLOAT) return fail(QBC_E_ARG, "qbc_upload: colour and normal buffers take GL_FLOAT data");
    if (itemsize != 12) return fail(QBC_E_ARG, "qbc_upload: colour/normal itemsize %zu (12 = one float3)", itemsize);
    const int64_t n_total = (int64_t)(size / 12);
    if (n_total > INT32_MAX) return fail(QBC_E_ARG, "qbc_upload: %lld points exceed int32 indices", (long long)n_total);
    DevModelBuf& m = c->model[(buftype == QBC_STATIC_COLOR || buftype == QBC_STATIC_NORMAL) ? 0 : 1];
    const bool is_col = buftype == QBC_STATIC_COLOR || buftype == QBC_DYNAMIC_COLOR;
    float4** arr = is_col ? &m.col : &m.nrm;
    int64_t* cap = is_col ? &m.cap_col : &m.cap_nrm;
    int64_t* n = is_col ? &m.n_col : &m.n_nrm;
    int64_t lo = (int64_t)(start / 12), hi = (int64_t)(end / 12);
    if (n_total > *cap) {
      int rc = grow(arr, cap, n_total + n_total / 8, 16, is_col ? "colour texels" : "normal texels");
      if (rc) return rc;
      lo = 0;
      hi = n_total;
    }
    *n = n_total;
    const int64_t chunk = (int64_t)(kStageMax / 12);
    if (hi > lo && !device_src) {
      int rc = ensure_stage(c, (size_t)std::min(hi - lo, chunk) * 12);
      if (rc) return rc;
    }
    for (int64_t a = lo; a < hi; a += chunk) {
      int64_t b = std::min(hi, a + chunk);
      const void* src = base + a * 12;
      if (!device_src) {
        QBC_CUDA(cudaMemcpyAsync(c->stage, src, (size_t)(b - a) * 12, cudaMemcpyHostToDevice, c->stream));
        src = c->stage;
      }
      qbc::expand_attr_kernel<<<launch_grid(c, b - a), 256, 0, c->stream>>>((const float*)src, b - a, *arr + a,
                                                                             1.0f);
      QBC_CUDA(cudaGetLastError());
      ++c->launches;
    }
  }
  QBC_CUDA(cudaStreamSynchronize(c->stream));
  return QBC_OK;
}
}  // namespace

// ---------------------------------------------------------------------------
// Rigid skinning of a character for the dynamic tree
// ---------------------------------------------------------------------------

namespace {

struct BoneSet {
  float m[QBC_MAX_BONES][12];  // row-major 3x3 rotation, then translation
};

__global__ void skin_rigid_kernel(const float* __restrict__ rp, const float* __restrict__ rn,
                                  const int32_t* __restrict__ bone, int64_t n, int n_bones,
                                  const __grid_constant__ BoneSet bones, float* __restrict__ op,
                                  float* __restrict__ on, int* __restrict__ bad) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    int b = bone[i];
    if (b < 0 || b >= n_bones) {
      atomicExch(bad, 1);
      b = 0;
    }
    const float* m = bones.m[b];
    const float x = rp[3 * i], y = rp[3 * i + 1], z = rp[3 * i + 2];
    op[3 * i] = m[0] * x + m[1] * y + m[2] * z + m[9];
    op[3 * i + 1] = m[3] * x + m[4] * y + m[5] * z + m[10];
    op[3 * i + 2] = m[6] * x + m[7] * y + m[8] * z + m[11];
    if (rn && on) {
      const float a = rn[3 * i], bb = rn[3 * i + 1], cc = rn[3 * i + 2];
      on[3 * i] = m[0] * a + m[1] * bb + m[2] * cc;
      on[3 * i + 1] = m[3] * a + m[4] * bb + m[5] * cc;
      on[3 * i + 2] = m[6] * a + m[7] * bb + m[8] * cc;
    }
  }
}

}  // namespace

extern "C" int qbc_skin_rigid(qbc_ctx* c, const float* rest_pnts, const float* rest_nrms, const int32_t* bone,
                              int64_t n, const float* bones, int n_bones, float* out_pnts, float* out_nrms) {
  qbc::clear_error();
  if (!c || (n > 0 && (!rest_pnts || !bone || !out_pnts)) || !bones)
    return fail(QBC_E_ARG, "qbc_skin_rigid: null argument");
  if (n_bones < 1 || n_bones > QBC_MAX_BONES)
    return fail(QBC_E_ARG, "qbc_skin_rigid: %d bones outside 1..%d", n_bones, QBC_MAX_BONES);
  if ((rest_nrms == nullptr) != (out_nrms == nullptr))
    return fail(QBC_E_ARG, "qbc_skin_rigid: give both normal arrays or neither");
  if (n == 0) return QBC_OK;
  QBC_CUDA(cudaSetDevice(c->device));
  BoneSet bs;
  std::memset(&bs, 0, sizeof(bs));
  std::memcpy(bs.m, bones, sizeof(float) * 12 * (size_t)n_bones);
  int rc = ensure_stage(c, 256);
  if (rc) return rc;
  int* bad = (int*)c->stage;
  QBC_CUDA(cudaMemsetAsync(bad, 0, sizeof(int), c->stream));
  skin_rigid_kernel<<<launch_grid(c, n), 256, 0, c->stream>>>(rest_pnts, rest_nrms, bone, n, n_bones, bs, out_pnts,
                                                              out_nrms, bad);
  QBC_CUDA(cudaGetLastError());
  ++c->launches;
  int hbad = 0;
  QBC_CUDA(cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  QBC_CUDA(cudaStreamSynchronize(c->stream));
  if (hbad) return fail(QBC_E_ARG, "qbc_skin_rigid: a bone index is outside 0..%d", n_bones - 1);
  return QBC_OK;
}

// ---------------------------------------------------------------------------
// GPU tree build (octree_insert_point / octree_insert_path order)
// ---------------------------------------------------------------------------

namespace {

int grow_tree_target(qbc::BuildTarget* t, int64_t nodes) {
  DevTreeBuf& tb = *static_cast<DevTreeBuf*>(t->user);
  if (nodes > tb.cap) {
    int64_t cap = nodes + nodes / 8;
    int rc = grow(&tb.child, &tb.cap, cap, 32, "octree child blocks");
    if (rc) return rc;
    int64_t mcap = 0;
    rc = grow(&tb.model, &mcap, cap, 4, "octree model indices");
    if (rc) return rc;
  }
  t->child = reinterpret_cast<int32_t*>(tb.child);
  t->model = tb.model;
  return QBC_OK;
}

int build_into(qbc_ctx* c, int tree, const float* pnts, const int32_t* octets, int64_t n, float basesize, int levels,
               int64_t first_index, int on_device) {
  if (!c || tree < 0 || tree > 1) return fail(QBC_E_ARG, "tree build: bad context or tree id");
  if (n < 0 || (n > 0 && !pnts && !octets)) return fail(QBC_E_ARG, "tree build: bad input");
  if (pnts && !(basesize > 0.0f)) return fail(QBC_E_ARG, "tree build: basesize must be positive");
  if (levels < 0 || levels > 21) return fail(QBC_E_ARG, "tree build: levels %d outside 0..21", levels);
  QBC_CUDA(cudaSetDevice(c->device));
  const float* dp = pnts;
  const int32_t* doc = octets;
  void* tmp = nullptr;
  if (!on_device && n > 0) {
    size_t bytes = pnts ? (size_t)n * 12 : (size_t)n * levels * 4;
    cudaError_t e = cudaMalloc(&tmp, bytes);
    if (e != cudaSuccess) return fail(QBC_E_NOMEM, "tree build input of %zu bytes: %s", bytes, cudaGetErrorString(e));
    e = cudaMemcpyAsync(tmp, pnts ? (const void*)pnts : (const void*)octets, bytes, cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) {
      cudaFree(tmp);
      return cuda_fail(e, "tree build input copy");
    }
    if (pnts)
      dp = static_cast<const float*>(tmp);
    else
      doc = static_cast<const int32_t*>(tmp);
  }
  qbc::BuildTarget t{nullptr, nullptr, 0, 0, &c->tree[tree], grow_tree_target};
  int rc = qbc::build_nodes(pnts ? dp : nullptr, pnts ? nullptr : doc, n, basesize, levels, first_index, c->stream, &t);
  if (tmp) cudaFree(tmp);
  c->launches += t.launches;
  if (rc) return rc;
  c->tree[tree].n = t.n_nodes;
  return QBC_OK;
}

__global__ void unpack_nodes_kernel(const int4* __restrict__ child, const int32_t* __restrict__ model, int64_t n,
                                    int4* __restrict__ raw) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    raw[3 * i] = child[2 * i];
    raw[3 * i + 1] = child[2 * i + 1];
    raw[3 * i + 2] = make_int4(model[i], 0, 0, 0);
  }
}

}  // namespace

extern "C" int qbc_build_tree(qbc_ctx* c, int tree, const float* pnts, int64_t n, float basesize, int levels,
                              int64_t first_index, int on_device) {
  qbc::clear_error();
  if (n > 0 && !pnts) return fail(QBC_E_ARG, "qbc_build_tree: null points");
  if (n == 0) pnts = reinterpret_cast<const float*>(&n);  // any non-null marker: no points to read
  return build_into(c, tree, pnts, nullptr, n, basesize, levels, first_index, on_device);
}

extern "C" int qbc_build_tree_paths(qbc_ctx* c, int tree, const int32_t* octets, int64_t n, int levels,
                                    int64_t first_index, int on_device) {
  qbc::clear_error();
  if (n > 0 && !octets) return fail(QBC_E_ARG, "qbc_build_tree_paths: null octets");
  if (n == 0) octets = reinterpret_cast<const int32_t*>(&n);
  return build_into(c, tree, nullptr, octets, n, 1.0f, levels, first_index, on_device);
}

extern "C" int qbc_load_flat(qbc_ctx* c, int tree, const char* pnt_path, const char* col_path, const char* nrm_path,
                             const char* rng_path, float basesize, int levels, int64_t* points, int64_t* nodes,
                             int32_t* ranges, int64_t range_cap, int64_t* range_ints) {
  qbc::clear_error();
  if (!c || tree < 0 || tree > 1) return fail(QBC_E_ARG, "qbc_load_flat: bad context or tree id");
  int64_t n = 0, nr = 0;
  int rc = qbc_flat_read(pnt_path, col_path, nrm_path, rng_path, nullptr, nullptr, nullptr, 0, &n, nullptr, 0, &nr);
  if (rc) return rc;
  std::vector<float> p, col, nrm;
  try {
    p.resize((size_t)n * 3);
    col.resize((size_t)n * 3);
    nrm.resize((size_t)n * 3);
  } catch (const std::bad_alloc&) {
    return fail(QBC_E_NOMEM, "qbc_load_flat: host arrays for %lld points", (long long)n);
  }
  rc = qbc_flat_read(pnt_path, col_path, nrm_path, rng_path, p.data(), col.data(), nrm.data(), n, &n, ranges,
                     range_cap, &nr);
  if (rc) return rc;
  // the reference's load: insert every point in file order, upload the
  // colours and normals as the tree's model (modelutil.c:180-255)
  const size_t bytes = (size_t)n * 12;
  if (n > 0) {
    rc = upload_impl(c, col.data(), QBC_GL_FLOAT, bytes, 12, 0, bytes, tree ? QBC_DYNAMIC_COLOR : QBC_STATIC_COLOR,
                     false);
    if (!rc)
      rc = upload_impl(c, nrm.data(), QBC_GL_FLOAT, bytes, 12, 0, bytes,
                       tree ? QBC_DYNAMIC_NORMAL : QBC_STATIC_NORMAL, false);
    if (rc) return rc;
  }
  const float* src = n > 0 ? p.data() : reinterpret_cast<const float*>(&n);
  rc = build_into(c, tree, src, nullptr, n, basesize, levels, 0, 0);
  if (rc) return rc;
  if (points) *points = n;
  if (nodes) *nodes = c->tree[tree].n;
  if (range_ints) *range_ints = nr;
  return QBC_OK;
}

extern "C" int qbc_tree_remove_points(qbc_ctx* c, int tree, const float* pts, int64_t n, float basesize, int levels,
                                      int on_device, int32_t* modind, int32_t* octind, int64_t* removed) {
  qbc::clear_error();
  if (!c || tree < 0 || tree > 1 || n < 0 || (n > 0 && !pts)) return fail(QBC_E_ARG, "qbc_tree_remove_points: bad argument");
  if (!(basesize > 0.0f) || levels < 0 || levels > QBC_MAX_LEVEL)
    return fail(QBC_E_ARG, "qbc_tree_remove_points: basesize > 0 and levels 0..%d required", QBC_MAX_LEVEL);
  if (c->tree[tree].n == 0) return fail(QBC_E_STATE, "qbc_tree_remove_points: no tree uploaded or built");
  QBC_CUDA(cudaSetDevice(c->device));
  if (n == 0) {
    if (removed) *removed = 0;
    return QBC_OK;
  }
  // device arrays: the caller's when on_device, else staged
  void* tmp = nullptr;
  const size_t pbytes = (size_t)n * 12, obytes = (size_t)n * 4;
  const float* dp = pts;
  int32_t* dm = modind;
  int32_t* dq = octind;
  const bool stage_out = !on_device || !modind || !octind;
  size_t need = (on_device ? 0 : pbytes) + (stage_out ? 2 * obytes : 0);
  if (need) {
    cudaError_t e = cudaMalloc(&tmp, need);
    if (e != cudaSuccess) return fail(QBC_E_NOMEM, "qbc_tree_remove_points: %s", cudaGetErrorString(e));
  }
  char* t = static_cast<char*>(tmp);
  int rc = QBC_OK;
  if (!on_device) {
    cudaError_t e = cudaMemcpyAsync(t, pts, pbytes, cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) rc = cuda_fail(e, "qbc_tree_remove_points: copy points");
    dp = reinterpret_cast<const float*>(t);
    t += pbytes;
  }
  if (stage_out) {
    dm = reinterpret_cast<int32_t*>(t);
    dq = reinterpret_cast<int32_t*>(t + obytes);
  }
  if (!rc)
    rc = qbc::remove_points(reinterpret_cast<int32_t*>(c->tree[tree].child), c->tree[tree].model, c->tree[tree].n,
                            dp, n, basesize, levels, dm, dq, removed, c->stream, &c->launches);
  if (!rc && stage_out) {
    // results to the caller's arrays (host, or device when only one was given)
    const cudaMemcpyKind k = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    cudaError_t e = cudaSuccess;
    if (modind) e = cudaMemcpyAsync(modind, dm, obytes, k, c->stream);
    if (e == cudaSuccess && octind) e = cudaMemcpyAsync(octind, dq, obytes, k, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) rc = cuda_fail(e, "qbc_tree_remove_points: copy results");
  }
  if (tmp) cudaFree(tmp);
  return rc;
}

extern "C" int qbc_download_tree(qbc_ctx* c, int tree, int32_t* nodes, int64_t cap, int64_t* n_nodes) {
  qbc::clear_error();
  if (!c || tree < 0 || tree > 1 || !n_nodes) return fail(QBC_E_ARG, "qbc_download_tree: bad argument");
  const int64_t n = c->tree[tree].n;
  *n_nodes = n;
  if (!nodes || n == 0) return QBC_OK;
  if (cap < n) return fail(QBC_E_ARG, "qbc_download_tree: capacity %lld below %lld nodes", (long long)cap, (long long)n);
  QBC_CUDA(cudaSetDevice(c->device));
  const int64_t chunk = (int64_t)(kStageMax / 48);
  int rc = ensure_stage(c, (size_t)std::min(n, chunk) * 48);
  if (rc) return rc;
  for (int64_t a = 0; a < n; a += chunk) {
    int64_t b = std::min(n, a + chunk);
    unpack_nodes_kernel<<<launch_grid(c, b - a), 256, 0, c->stream>>>(c->tree[tree].child + 2 * a,
                                                                       c->tree[tree].model + a, b - a,
                                                                       (int4*)c->stage);
    QBC_CUDA(cudaGetLastError());
    ++c->launches;
    QBC_CUDA(cudaMemcpyAsync(nodes + a * 12, c->stage, (size_t)(b - a) * 48, cudaMemcpyDeviceToHost, c->stream));
  }
  QBC_CUDA(cudaStreamSynchronize(c->stream));
  return QBC_OK;
}

// ---------------------------------------------------------------------------
// Occluder-proposal network: features, dataset, training, inference
// ---------------------------------------------------------------------------

namespace {

using bf16 = __nv_bfloat16;

// Network input of a shade-pass record: hit point normalised to the
// basecube, unit normal, unit direction to the light, and sin/cos of pi
// times the normalised hit point scaled by 4, 8, ..., 128 (45 values, zero
// padded).
__device__ __forceinline__ void record_features(const qbc::Batch& b, const uint32_t* r, bf16* x) {
  const qbc_view& v = b.job[r[qbc::kPxView]].v;
  const float S = v.basecube[3];
  const float lo[3] = {v.basecube[0], v.basecube[1] - S, v.basecube[2] - S};
  float f[qbc::mlp::kIn];
  float isp[3], n[3], l[3];
  for (int k = 0; k < 3; ++k) {
    isp[k] = __uint_as_float(r[qbc::kPxIsp + k]);
    n[k] = __uint_as_float(r[qbc::kPxNrm + k]);
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
__global__ void collect_kernel(const __grid_constant__ qbc::Batch b, const __grid_constant__ qbc::Wave w,
                               bf16* __restrict__ X, float* __restrict__ tl, int8_t* __restrict__ kind,
                               unsigned int* __restrict__ count, int64_t cap) {
  const unsigned total = min(*w.qcount, w.cap);
  for (unsigned q = blockIdx.x * blockDim.x + threadIdx.x; q < total; q += gridDim.x * blockDim.x) {
    const uint32_t* r = w.rec + (size_t)q * qbc::kRecWords;
    if (!(r[qbc::kPxFlags] & QBC_PX_SHADED)) continue;
    const float t = __uint_as_float(r[qbc::kRecLogT]);
    const bool lit = r[qbc::kRecLogLit] != 0;
    const bool occluded = !lit && t > 0.0f && t < 1.0f;
    if (!lit && !occluded) continue;  // unlit without an occluder before the hit: no label
    const unsigned i = atomicAdd(count, 1u);
    if ((int64_t)i >= cap) continue;
    record_features(b, r, X + (size_t)i * qbc::mlp::kIn);
    tl[i] = occluded ? t : 2.0f;
    kind[i] = occluded ? 1 : 0;
  }
}

// Fused-network rows over the shade-pass record queue: the features of each
// record in, its proposals out (earliest first; none where the occlusion
// logit is below the gate). The row count is read on the device.
struct RecordRows {
  qbc::Batch b;
  qbc::Wave w;
  float gate;
  int keep;  // proposals kept, earliest first
  __device__ __forceinline__ uint32_t rows() const { return min(*w.qcount, w.cap); }
  __device__ __forceinline__ void load(uint32_t r0, uint32_t n, bf16* x, int lane) const {
    if (lane >= 16) return;
    bf16* row = x + lane * qbc::mlp::kLdIn;
    if ((uint32_t)lane < n) {
      record_features(b, w.rec + (size_t)(r0 + lane) * qbc::kRecWords, row);
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

// One launch of the fused network over `src`'s rows: a persistent grid of
// resident blocks, each staging the weights once.
template <class Src>
int launch_fused(qbc_ctx* c, const Src& src, int variant) {
  using qbc::mlp::FusedSmem;
  auto kern = qbc::mlp::fused_forward_kernel<Src>;
  if (!c->fused_attr[variant]) {
    QBC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(FusedSmem)));
    c->fused_attr[variant] = true;
  }
  int per_sm = 0;
  QBC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, qbc::mlp::kFusedThreads, sizeof(FusedSmem)));
  if (per_sm < 1) return fail(QBC_E_STATE, "proposal network: no block fits on an SM");
  qbc::mlp::FusedParams p;
  for (int l = 0; l < 4; ++l) {
    p.w[l] = c->net.wb + qbc::mlp::param_offset(l, false);
    p.b[l] = c->net.master + qbc::mlp::param_offset(l, true);
    if (reinterpret_cast<uintptr_t>(p.w[l]) % 16) return fail(QBC_E_STATE, "proposal network: unaligned weights");
  }
  kern<<<per_sm * c->sm_count, qbc::mlp::kFusedThreads, sizeof(FusedSmem), c->stream>>>(p, src);
  QBC_CUDA(cudaGetLastError());
  ++c->launches;
  return QBC_OK;
}

// Proposals of every queued record from the network (no host round trip:
// the kernel reads the queue length on the device).
int propose_mlp(qbc_ctx* c, const qbc::Batch& b, const qbc::Wave& w) {
  if (!c->net.ready) return fail(QBC_E_STATE, "qbc_render_views_ex: no occluder network in this context");
  std::unique_ptr<RecordRows> src(new RecordRows());
  src->b = b;
  src->w = w;
  const float p = (float)c->proposal_gate * 1e-3f;  // gate probability -> logit
  src->gate = c->proposal_gate <= 0 ? -INFINITY : logf(p / (1.0f - p));
  src->keep = c->proposal_count;
  return launch_fused(c, *src, 0);
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

// ---------------------------------------------------------------------------
// Render
// ---------------------------------------------------------------------------

namespace {

int check_view(const qbc_view& v, int i) {
  if (v.width_px < 1 || v.height_px < 1 || v.width_px > 65536 || v.height_px > 65536)
    return fail(QBC_E_ARG, "view %d: %dx%d pixels outside 1..65536", i, v.width_px, v.height_px);
  if (v.maxlevel < 0 || v.maxlevel > QBC_MAX_LEVEL)
    return fail(QBC_E_ARG, "view %d: maxlevel %d outside 0..%d", i, v.maxlevel, QBC_MAX_LEVEL);
  return QBC_OK;
}

// Bytes per pixel of each output stream, in qbc_outputs order.
constexpr size_t kOutBytes[6] = {4, 16, 4, 16, 16, 16};

void** out_slot(qbc_outputs& o, int k) {
  switch (k) {
    case 0: return (void**)&o.rgba8;
    case 1: return (void**)&o.rgba32f;
    case 2: return (void**)&o.flags;
    case 3: return (void**)&o.leaf;
    case 4: return (void**)&o.isp;
    default: return (void**)&o.visits;
  }
}

int propose_mlp(qbc_ctx* c, const qbc::Batch& b, const qbc::Wave& w);

// Statistics of the shade passes of the last two-pass render (synchronizes).
int read_stats(qbc_ctx* c, qbc_render_stats* stats) {
  if (!stats) return QBC_OK;
  unsigned long long h[qbc::kStatCount];
  unsigned int q[2];
  QBC_CUDA(cudaMemcpyAsync(h, c->wstats, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  QBC_CUDA(cudaMemcpyAsync(q, c->wcount, sizeof(q), cudaMemcpyDeviceToHost, c->stream));
  QBC_CUDA(cudaStreamSynchronize(c->stream));
  stats->queued = q[0];
  stats->shadow_rays = h[qbc::kStatShadowRays];
  stats->shadow_visits = h[qbc::kStatShadowVisits];
  stats->proposals_tried = h[qbc::kStatPropTried];
  stats->proposals_proven = h[qbc::kStatPropProven];
  stats->proposal_visits = h[qbc::kStatPropVisits];
  return QBC_OK;
}

template <bool EXACT, bool DYN, int MODE, bool PROP>
int launch_render(qbc_ctx* c, const qbc::Batch& b, size_t smem, const qbc::Wave& wave) {
  auto kern = qbc::render_kernel<EXACT, DYN, MODE, PROP>;
  const int variant = (EXACT ? 1 : 0) + (DYN ? 2 : 0) + 4 * MODE + (PROP ? 16 : 0);
  if (!(c->attr_done & (1 << variant))) {
    QBC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024));
    c->attr_done |= 1 << variant;
  }
  int per_sm = 0;
  QBC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, qbc::kThreads, smem));
  if (per_sm < 1) return fail(QBC_E_STATE, "render_kernel: no block fits on an SM with %zu B shared memory", smem);
  if (MODE == qbc::kFused && !PROP) c->render_blocks[(EXACT ? 1 : 0) + (DYN ? 2 : 0)] = per_sm;
  if (c->blocks_per_sm > 0) per_sm = std::min(per_sm, c->blocks_per_sm);
  // persistent: one wave of resident blocks, never more blocks than warp tiles
  int64_t blocks = (int64_t)per_sm * c->sm_count;
  if (MODE != qbc::kShadePass) blocks = std::min<int64_t>(blocks, ((int64_t)b.tiles_total + 3) / 4);
  blocks = std::max<int64_t>(blocks, 1);
  if (MODE != qbc::kShadePass) QBC_CUDA(cudaMemsetAsync(c->queue, 0, sizeof(unsigned int), c->stream));
  kern<<<(unsigned)blocks, qbc::kThreads, smem, c->stream>>>(device_scene(c), b, c->queue, wave);
  QBC_CUDA(cudaGetLastError());
  ++c->launches;
  return QBC_OK;
}

template <bool EXACT, bool DYN>
int launch_modes(qbc_ctx* c, const qbc::Batch& b, size_t smem, const qbc_render_opts* opts, int64_t pixels) {
  if (!opts || !opts->two_pass) return launch_render<EXACT, DYN, qbc::kFused, false>(c, b, smem, qbc::Wave{});
  // two passes: primary rays -> record queue -> shade pass
  if (c->rec_cap < pixels) {
    int rc = grow(&c->rec, &c->rec_cap, pixels, (size_t)qbc::kRecWords * 4, "render records");
    if (rc) return rc;
  }
  const bool want_log = opts->log || opts->proposals == QBC_PROPOSE_LOGGED;
  if (want_log && c->pixlog_cap < pixels) {
    int rc = grow(&c->pixlog, &c->pixlog_cap, pixels, 4, "render log");
    if (rc) return rc;
  }
  if (opts->proposals == QBC_PROPOSE_LOGGED && c->pixlog_valid != pixels)
    return fail(QBC_E_STATE, "qbc_render_views_ex: logged proposals need a logged render of the same views first");
  qbc::Wave w{};
  w.rec = c->rec;
  w.qcount = c->wcount;
  w.qnext = c->wcount + 1;
  w.stats = c->wstats;
  w.cap = (uint32_t)std::min<int64_t>(c->rec_cap, 0xFFFFFFFFll);
  w.log = opts->log ? 1 : 0;
  w.nprop = opts->proposals != QBC_PROPOSE_NONE ? 3 : 0;
  w.pdepth = opts->proposal_level > 0 ? opts->proposal_level : 8;
  w.pixlog = opts->log ? c->pixlog : nullptr;
  QBC_CUDA(cudaMemsetAsync(c->wcount, 0, 2 * sizeof(unsigned int), c->stream));
  int rc = launch_render<EXACT, DYN, qbc::kPrimaryPass, false>(c, b, smem, w);
  if (rc) return rc;
  if (opts->proposals == QBC_PROPOSE_LOGGED) {
    qbc::Wave lw = w;
    lw.pixlog = c->pixlog;
    qbc::fill_logged_proposals<<<c->sm_count * 8, 256, 0, c->stream>>>(b, lw);
    QBC_CUDA(cudaGetLastError());
    ++c->launches;
  } else if (opts->proposals == QBC_PROPOSE_RANDOM) {
    qbc::fill_random_proposals<<<c->sm_count * 8, 256, 0, c->stream>>>(w, (unsigned long long)opts->seed);
    QBC_CUDA(cudaGetLastError());
    ++c->launches;
  } else if (opts->proposals == QBC_PROPOSE_MLP) {
    rc = propose_mlp(c, b, w);
    if (rc) return rc;
  }
  if (w.nprop > 0) rc = launch_render<EXACT, DYN, qbc::kShadePass, true>(c, b, smem, w);
  else rc = launch_render<EXACT, DYN, qbc::kShadePass, false>(c, b, smem, w);
  if (rc) return rc;
  if (opts->log) c->pixlog_valid = pixels;
  return QBC_OK;
}

int launch_batch(qbc_ctx* c, const qbc_view* views, const qbc_outputs* dev_outs, int n,
                 const qbc_render_opts* opts = nullptr) {
  qbc::Batch* b = new qbc::Batch();
  int tiles = 0, maxlevel = 0;
  int64_t pixels = 0;
  bool exact = true;
  for (int i = 0; i < n; ++i) {
    qbc::ViewJob& J = b->job[i];
    J.v = views[i];
    J.o = dev_outs[i];
    const int tw = 1 << c->tile_shift, th = 32 >> c->tile_shift;
    J.tiles_x = (views[i].width_px + tw - 1) / tw;
    int tiles_y = (views[i].height_px + th - 1) / th;
    J.tile_begin = tiles;
    J.pixel_begin = pixels;
    tiles += J.tiles_x * tiles_y;
    pixels += (int64_t)views[i].width_px * views[i].height_px;
    maxlevel = std::max(maxlevel, views[i].maxlevel);
    exact = exact && qbc::cube_shift_exact(views[i]);
  }
  b->n = n;
  b->tiles_total = tiles;
  b->max_level = maxlevel;
  b->service_min = c->service_min;
  b->tile_shift = c->tile_shift;
  const bool dyn = c->tree[1].n > 0;
  const size_t words = (size_t)(dyn ? 3 : 2) * maxlevel + qbc::kPixWords;
  const size_t smem = words * qbc::kThreads * sizeof(uint32_t);
  int rc;
  if (exact)
    rc = dyn ? launch_modes<true, true>(c, *b, smem, opts, pixels) : launch_modes<true, false>(c, *b, smem, opts, pixels);
  else
    rc = dyn ? launch_modes<false, true>(c, *b, smem, opts, pixels) : launch_modes<false, false>(c, *b, smem, opts, pixels);
  delete b;
  return rc;
}

}  // namespace

namespace {
int render_views_impl(qbc_ctx* c, const qbc_view* views, const qbc_outputs* outs, int n, int outputs_on_device,
                      const qbc_render_opts* opts, qbc_render_stats* stats);
int check_render_opts(const qbc_render_opts* opts, int n);
}

extern "C" int qbc_render_views(qbc_ctx* c, const qbc_view* views, const qbc_outputs* outs, int n,
                                int outputs_on_device) {
  qbc::clear_error();
  return render_views_impl(c, views, outs, n, outputs_on_device, nullptr, nullptr);
}

extern "C" int qbc_render_views_ex(qbc_ctx* c, const qbc_view* views, const qbc_outputs* outs, int n,
                                   int outputs_on_device, const qbc_render_opts* opts, qbc_render_stats* stats) {
  qbc::clear_error();
  int rc = check_render_opts(opts, n);
  if (rc) return rc;
  return render_views_impl(c, views, outs, n, outputs_on_device, opts, stats);
}

namespace {
int render_views_impl(qbc_ctx* c, const qbc_view* views, const qbc_outputs* outs, int n, int outputs_on_device,
                      const qbc_render_opts* opts, qbc_render_stats* stats) {
  if (!c || (n > 0 && (!views || !outs))) return fail(QBC_E_ARG, "qbc_render_views: null argument");
  if (n < 0) return fail(QBC_E_ARG, "qbc_render_views: negative view count");
  QBC_CUDA(cudaSetDevice(c->device));
  for (int i = 0; i < n; ++i) {
    int rc = check_view(views[i], i);
    if (rc) return rc;
  }

  const bool two = opts && opts->two_pass;
  if (two) QBC_CUDA(cudaMemsetAsync(c->wstats, 0, qbc::kStatCount * sizeof(unsigned long long), c->stream));
  if (outputs_on_device) {
    for (int a = 0; a < n; a += qbc::kMaxViewsPerLaunch) {
      int rc = launch_batch(c, views + a, outs + a, std::min(qbc::kMaxViewsPerLaunch, n - a), opts);
      if (rc) return rc;
    }
    return two ? read_stats(c, stats) : QBC_OK;
  }

  // host outputs: render into device scratch, then copy each stream back
  std::vector<qbc_outputs> dev(n);
  size_t need = 0;
  for (int i = 0; i < n; ++i) {
    size_t px = (size_t)views[i].width_px * views[i].height_px;
    qbc_outputs h = outs[i];
    for (int k = 0; k < 6; ++k)
      if (*out_slot(h, k)) need += (px * kOutBytes[k] + 255) & ~size_t(255);
  }
  if (need > c->scratch_bytes) {
    if (c->scratch) QBC_CUDA(cudaFree(c->scratch));
    c->scratch = nullptr;
    c->scratch_bytes = 0;
    cudaError_t e = cudaMalloc(&c->scratch, need);
    if (e != cudaSuccess) return fail(QBC_E_NOMEM, "render scratch of %zu bytes: %s", need, cudaGetErrorString(e));
    c->scratch_bytes = need;
  }
  size_t off = 0;
  for (int i = 0; i < n; ++i) {
    size_t px = (size_t)views[i].width_px * views[i].height_px;
    qbc_outputs h = outs[i];
    std::memset(&dev[i], 0, sizeof(qbc_outputs));
    for (int k = 0; k < 6; ++k) {
      if (!*out_slot(h, k)) continue;
      *out_slot(dev[i], k) = (char*)c->scratch + off;
      off += (px * kOutBytes[k] + 255) & ~size_t(255);
    }
  }
  for (int a = 0; a < n; a += qbc::kMaxViewsPerLaunch) {
    int rc = launch_batch(c, views + a, dev.data() + a, std::min(qbc::kMaxViewsPerLaunch, n - a), opts);
    if (rc) return rc;
  }
  for (int i = 0; i < n; ++i) {
    size_t px = (size_t)views[i].width_px * views[i].height_px;
    qbc_outputs h = outs[i];
    for (int k = 0; k < 6; ++k) {
      void* dst = *out_slot(h, k);
      if (!dst) continue;
      QBC_CUDA(cudaMemcpyAsync(dst, *out_slot(dev[i], k), px * kOutBytes[k], cudaMemcpyDeviceToHost, c->stream));
    }
  }
  QBC_CUDA(cudaStreamSynchronize(c->stream));
  return two ? read_stats(c, stats) : QBC_OK;
}
}  // namespace

// ---------------------------------------------------------------------------
// A frame as a CUDA graph
// ---------------------------------------------------------------------------

namespace {

// Everything a captured frame bakes into its kernel parameters besides the
// views: device addresses and sizes of the trees, models and work buffers,
// and the options that become launch parameters.
struct FrameSignature {
  qbc::DevScene scene;
  const void* rec;
  int64_t rec_cap;
  const void* pixlog;
  int64_t pixlog_cap;
  const void* net_w;
  const void* net_b;
  const void* stream;
  int32_t service_min;
  int32_t proposal_gate;
  int32_t tile_shift;
  int32_t blocks_per_sm;
  int32_t proposal_count;
};

bool same_signature(const FrameSignature& a, const FrameSignature& b) {
  for (int t = 0; t < 2; ++t) {
    const qbc::DevTree &ta = a.scene.tree[t], &tb = b.scene.tree[t];
    const qbc::DevModel &ma = a.scene.model[t], &mb = b.scene.model[t];
    if (ta.child != tb.child || ta.model != tb.model || ta.n != tb.n) return false;
    if (ma.col != mb.col || ma.nrm != mb.nrm || ma.n != mb.n) return false;
  }
  return a.rec == b.rec && a.rec_cap == b.rec_cap && a.pixlog == b.pixlog && a.pixlog_cap == b.pixlog_cap &&
         a.net_w == b.net_w && a.net_b == b.net_b && a.stream == b.stream && a.service_min == b.service_min &&
         a.proposal_gate == b.proposal_gate && a.tile_shift == b.tile_shift && a.blocks_per_sm == b.blocks_per_sm &&
         a.proposal_count == b.proposal_count;
}

FrameSignature frame_signature(const qbc_ctx* c) {
  FrameSignature f;
  f.scene = device_scene(c);
  f.rec = c->rec;
  f.rec_cap = c->rec_cap;
  f.pixlog = c->pixlog;
  f.pixlog_cap = c->pixlog_cap;
  f.net_w = c->net.wb;
  f.net_b = c->net.master;
  f.stream = c->stream;
  f.service_min = c->service_min;
  f.proposal_gate = c->proposal_gate;
  f.tile_shift = c->tile_shift;
  f.blocks_per_sm = c->blocks_per_sm;
  f.proposal_count = c->proposal_count;
  return f;
}

int check_render_opts(const qbc_render_opts* opts, int n) {
  if (opts && (opts->proposals < QBC_PROPOSE_NONE || opts->proposals > QBC_PROPOSE_RANDOM))
    return fail(QBC_E_ARG, "qbc_render_views_ex: unknown proposal source %d", opts->proposals);
  if (opts && opts->proposals != QBC_PROPOSE_NONE && !opts->two_pass)
    return fail(QBC_E_ARG, "qbc_render_views_ex: proposals need two_pass");
  if (opts && (opts->proposal_level < 0 || opts->proposal_level > QBC_MAX_LEVEL))
    return fail(QBC_E_ARG, "qbc_render_views_ex: proposal_level %d outside 0..%d", opts->proposal_level, QBC_MAX_LEVEL);
  if (opts && opts->two_pass && n > qbc::kMaxViewsPerLaunch)
    return fail(QBC_E_ARG, "qbc_render_views_ex: two-pass renders take at most %d views per call", qbc::kMaxViewsPerLaunch);
  return QBC_OK;
}

}  // namespace

struct qbc_graph {
  qbc_ctx* ctx = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<qbc_outputs> outs;
  std::vector<int32_t> sizes;  // width, height per view
  qbc_render_opts opts;
  bool has_opts = false;
  int n = 0;
  int64_t kernels = 0;
  FrameSignature sig;
};

namespace {

int capture_frame(qbc_graph* g, const qbc_view* views, cudaGraph_t* out) {
  qbc_ctx* c = g->ctx;
  QBC_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  const int rc = render_views_impl(c, views, g->outs.data(), g->n, 1, g->has_opts ? &g->opts : nullptr, nullptr);
  cudaGraph_t graph = nullptr;
  const cudaError_t e = cudaStreamEndCapture(c->stream, &graph);
  if (rc || e != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    cudaGetLastError();
    return rc ? rc : cuda_fail(e, "frame capture");
  }
  *out = graph;
  return QBC_OK;
}

int64_t kernel_nodes(cudaGraph_t graph) {
  size_t n = 0;
  if (cudaGraphGetNodes(graph, nullptr, &n) != cudaSuccess) return 0;
  std::vector<cudaGraphNode_t> nodes(n);
  if (n && cudaGraphGetNodes(graph, nodes.data(), &n) != cudaSuccess) return 0;
  int64_t k = 0;
  for (cudaGraphNode_t node : nodes) {
    cudaGraphNodeType t;
    if (cudaGraphNodeGetType(node, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++k;
  }
  return k;
}

void release_graph(qbc_graph* g) {
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  g->exec = nullptr;
  g->graph = nullptr;
}

}  // namespace

// The context is going: free the graph's CUDA objects; the handle stays
// valid for qbc_graph_destroy and fails every other call.
void detach_graph(qbc_graph* g) {
  release_graph(g);
  g->ctx = nullptr;
}

extern "C" int qbc_graph_capture(qbc_ctx* c, const qbc_view* views, const qbc_outputs* dev_outs, int n,
                                 const qbc_render_opts* opts, qbc_graph** out) {
  qbc::clear_error();
  if (!c || !views || !dev_outs || !out || n <= 0) return fail(QBC_E_ARG, "qbc_graph_capture: bad argument");
  int rc = check_render_opts(opts, n);
  if (rc) return rc;
  QBC_CUDA(cudaSetDevice(c->device));
  // one eager frame first: buffers grown and kernel attributes set before
  // the capture, which must not allocate
  rc = render_views_impl(c, views, dev_outs, n, 1, opts, nullptr);
  if (rc) return rc;
  QBC_CUDA(cudaStreamSynchronize(c->stream));
  std::unique_ptr<qbc_graph> g(new qbc_graph());
  g->ctx = c;
  g->n = n;
  g->outs.assign(dev_outs, dev_outs + n);
  for (int i = 0; i < n; ++i) {
    g->sizes.push_back(views[i].width_px);
    g->sizes.push_back(views[i].height_px);
  }
  std::memset(&g->opts, 0, sizeof(g->opts));
  if (opts) {
    g->opts = *opts;
    g->has_opts = true;
  }
  g->sig = frame_signature(c);
  rc = capture_frame(g.get(), views, &g->graph);
  if (rc) return rc;
  cudaError_t e = cudaGraphInstantiate(&g->exec, g->graph, 0);
  if (e != cudaSuccess) {
    release_graph(g.get());
    return cuda_fail(e, "qbc_graph_capture: instantiate");
  }
  g->kernels = kernel_nodes(g->graph);
  c->graphs.push_back(g.get());
  *out = g.release();
  return QBC_OK;
}

extern "C" int qbc_graph_update(qbc_graph* g, const qbc_view* views, int n) {
  qbc::clear_error();
  if (!g || !views || n != g->n) return fail(QBC_E_ARG, "qbc_graph_update: bad argument (views must match the capture)");
  if (!g->ctx) return fail(QBC_E_STATE, "qbc_graph_update: the graph's context was destroyed");
  for (int i = 0; i < n; ++i)
    if (views[i].width_px != g->sizes[2 * i] || views[i].height_px != g->sizes[2 * i + 1])
      return fail(QBC_E_ARG, "qbc_graph_update: view %d is %dx%d, captured %dx%d", i, views[i].width_px,
                  views[i].height_px, g->sizes[2 * i], g->sizes[2 * i + 1]);
  qbc_ctx* c = g->ctx;
  QBC_CUDA(cudaSetDevice(c->device));
  g->sig = frame_signature(c);
  cudaGraph_t fresh = nullptr;
  int rc = capture_frame(g, views, &fresh);
  if (rc) return rc;
  cudaGraphExecUpdateResultInfo info;
  if (cudaGraphExecUpdate(g->exec, fresh, &info) != cudaSuccess) {
    // a different topology (e.g. another kernel variant): instantiate anew
    cudaGetLastError();
    cudaGraphExec_t exec = nullptr;
    cudaError_t e = cudaGraphInstantiate(&exec, fresh, 0);
    if (e != cudaSuccess) {
      cudaGraphDestroy(fresh);
      return cuda_fail(e, "qbc_graph_update: instantiate");
    }
    cudaGraphExecDestroy(g->exec);
    g->exec = exec;
  }
  cudaGraphDestroy(g->graph);
  g->graph = fresh;
  g->kernels = kernel_nodes(fresh);
  return QBC_OK;
}

extern "C" int qbc_graph_launch(qbc_graph* g) {
  qbc::clear_error();
  if (!g) return fail(QBC_E_ARG, "qbc_graph_launch: null graph");
  if (!g->ctx || !g->exec) return fail(QBC_E_STATE, "qbc_graph_launch: the graph's context was destroyed");
  qbc_ctx* c = g->ctx;
  if (!same_signature(frame_signature(c), g->sig))
    return fail(QBC_E_STATE, "qbc_graph_launch: scene, buffers, stream or options changed since the capture "
                             "(qbc_graph_update re-captures)");
  QBC_CUDA(cudaSetDevice(c->device));
  QBC_CUDA(cudaGraphLaunch(g->exec, c->stream));
  c->launches += g->kernels;
  return QBC_OK;
}

extern "C" int qbc_graph_destroy(qbc_graph* g) {
  if (!g) return QBC_OK;
  if (qbc_ctx* c = g->ctx) {
    cudaSetDevice(c->device);
    c->graphs.erase(std::remove(c->graphs.begin(), c->graphs.end(), g), c->graphs.end());
  }
  release_graph(g);
  delete g;
  return QBC_OK;
}

// ---------------------------------------------------------------------------
// Autotuner: service threshold, warp tile width, render blocks per SM
// ---------------------------------------------------------------------------

namespace {

struct TuneSetting {
  int shift, blocks, service;
};

// Median device time of `reps` frames (after one untimed frame).
int time_frames(qbc_ctx* c, const qbc_view* views, const qbc_outputs* outs, int n, const qbc_render_opts* opts,
                int reps, cudaEvent_t* ev, float* ms) {
  int rc = render_views_impl(c, views, outs, n, 1, opts, nullptr);
  if (rc) return rc;
  std::vector<float> t((size_t)reps);
  for (int r = 0; r < reps; ++r) {
    QBC_CUDA(cudaEventRecord(ev[0], c->stream));
    rc = render_views_impl(c, views, outs, n, 1, opts, nullptr);
    if (rc) return rc;
    QBC_CUDA(cudaEventRecord(ev[1], c->stream));
    QBC_CUDA(cudaEventSynchronize(ev[1]));
    QBC_CUDA(cudaEventElapsedTime(&t[(size_t)r], ev[0], ev[1]));
  }
  std::sort(t.begin(), t.end());
  *ms = t[(size_t)reps / 2];
  return QBC_OK;
}

int autotune_impl(qbc_ctx* c, const qbc_view* views, const qbc_outputs* outs, int n, const qbc_render_opts* opts,
                  int reps, cudaEvent_t* ev, TuneSetting* best, qbc_tune_result* res) {
  auto apply = [c](const TuneSetting& s) {
    c->tile_shift = s.shift;
    c->blocks_per_sm = s.blocks;
    c->service_min = s.service;
  };
  float best_ms = 0.0f;
  int rc = time_frames(c, views, outs, n, opts, reps, ev, &best_ms);
  if (rc) return rc;
  res->ms_initial = best_ms;
  res->candidates = 1;
  auto consider = [&](const TuneSetting& s) -> int {
    apply(s);
    float ms = 0.0f;
    int e = time_frames(c, views, outs, n, opts, reps, ev, &ms);
    if (e) return e;
    ++res->candidates;
    if (ms < best_ms) {
      best_ms = ms;
      *best = s;
    }
    return QBC_OK;
  };
  // one option at a time, each kept at its best before the next is swept
  for (int sm : {1, 2, 3, 4, 6, 8, 12, 16})
    if (sm != best->service && (rc = consider({best->shift, best->blocks, sm}))) return rc;
  for (int sh : {1, 2, 3, 4, 5})
    if (sh != best->shift && (rc = consider({sh, best->blocks, best->service}))) return rc;
  for (int bl : {0, 2, 3, 4, 6, 8})
    if (bl != best->blocks && (rc = consider({best->shift, bl, best->service}))) return rc;
  res->ms_best = best_ms;
  return QBC_OK;
}

}  // namespace

extern "C" int qbc_autotune(qbc_ctx* c, const qbc_view* views, const qbc_outputs* dev_outs, int n,
                            const qbc_render_opts* opts, int reps, qbc_tune_result* result) {
  qbc::clear_error();
  if (!c || !views || !dev_outs || !result || n <= 0) return fail(QBC_E_ARG, "qbc_autotune: bad argument");
  if (reps < 1 || reps > 101) return fail(QBC_E_ARG, "qbc_autotune: reps %d outside 1..101", reps);
  int rc = check_render_opts(opts, n);
  if (rc) return rc;
  QBC_CUDA(cudaSetDevice(c->device));
  std::memset(result, 0, sizeof(*result));
  cudaEvent_t ev[2] = {nullptr, nullptr};
  QBC_CUDA(cudaEventCreate(&ev[0]));
  if (cudaEventCreate(&ev[1]) != cudaSuccess) {
    cudaEventDestroy(ev[0]);
    return fail(QBC_E_CUDA, "qbc_autotune: event");
  }
  const TuneSetting initial{c->tile_shift, c->blocks_per_sm, c->service_min};
  TuneSetting best = initial;
  rc = autotune_impl(c, views, dev_outs, n, opts, reps, ev, &best, result);
  const TuneSetting keep = rc ? initial : best;
  c->tile_shift = keep.shift;
  c->blocks_per_sm = keep.blocks;
  c->service_min = keep.service;
  cudaEventDestroy(ev[0]);
  cudaEventDestroy(ev[1]);
  if (rc) return rc;
  result->tile_width = 1 << keep.shift;
  result->blocks_per_sm = keep.blocks;
  result->service_min = keep.service;
  return QBC_OK;
}

extern "C" int qbc_trace_rays(qbc_ctx* c, const float* pos, const float* dir, int64_t n, const float basecube[4],
                              int maxlevel, const qbc_ray_hits* out, int on_device) {
  qbc::clear_error();
  if (!c || !basecube || !out || (n > 0 && (!pos || !dir))) return fail(QBC_E_ARG, "qbc_trace_rays: null argument");
  if (n < 0) return fail(QBC_E_ARG, "qbc_trace_rays: negative ray count");
  if (maxlevel < 0 || maxlevel > QBC_MAX_LEVEL)
    return fail(QBC_E_ARG, "qbc_trace_rays: maxlevel %d outside 0..%d", maxlevel, QBC_MAX_LEVEL);
  if (n == 0) return QBC_OK;
  QBC_CUDA(cudaSetDevice(c->device));
  qbc_view probe;
  std::memset(&probe, 0, sizeof(probe));
  for (int k = 0; k < 4; ++k) probe.basecube[k] = basecube[k];
  probe.maxlevel = maxlevel;
  qbc::RayJob job;
  job.n = n;
  job.bc = make_float4(basecube[0], basecube[1], basecube[2], basecube[3]);
  job.maxlevel = maxlevel;
  // per-ray bytes of each output, in qbc_ray_hits order
  const size_t bytes[7] = {4, 8, 8, 16, 16, 16, 8};
  void* const* hs[7] = {(void* const*)&out->status, (void* const*)&out->leaf, (void* const*)&out->model,
                        (void* const*)&out->isp,    (void* const*)&out->col,  (void* const*)&out->nrm,
                        (void* const*)&out->visits};
  void* dv[7] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  if (on_device) {
    job.pos = pos;
    job.dir = dir;
    for (int k = 0; k < 7; ++k) dv[k] = *hs[k];
  } else {
    size_t need = 2 * ((size_t)n * 12 + 256);
    for (int k = 0; k < 7; ++k)
      if (*hs[k]) need += ((size_t)n * bytes[k] + 255) & ~size_t(255);
    if (need > c->scratch_bytes) {
      if (c->scratch) QBC_CUDA(cudaFree(c->scratch));
      c->scratch = nullptr;
      c->scratch_bytes = 0;
      cudaError_t e = cudaMalloc(&c->scratch, need);
      if (e != cudaSuccess) return fail(QBC_E_NOMEM, "ray scratch of %zu bytes: %s", need, cudaGetErrorString(e));
      c->scratch_bytes = need;
    }
    char* base = (char*)c->scratch;
    size_t off = 0;
    float* dpos = (float*)(base + off);
    off += ((size_t)n * 12 + 255) & ~size_t(255);
    float* ddir = (float*)(base + off);
    off += ((size_t)n * 12 + 255) & ~size_t(255);
    for (int k = 0; k < 7; ++k) {
      if (!*hs[k]) continue;
      dv[k] = base + off;
      off += ((size_t)n * bytes[k] + 255) & ~size_t(255);
    }
    QBC_CUDA(cudaMemcpyAsync(dpos, pos, (size_t)n * 12, cudaMemcpyHostToDevice, c->stream));
    QBC_CUDA(cudaMemcpyAsync(ddir, dir, (size_t)n * 12, cudaMemcpyHostToDevice, c->stream));
    job.pos = dpos;
    job.dir = ddir;
  }
  job.o.status = (int32_t*)dv[0];
  job.o.leaf = (int32_t*)dv[1];
  job.o.model = (int32_t*)dv[2];
  job.o.isp = (float*)dv[3];
  job.o.col = (float*)dv[4];
  job.o.nrm = (float*)dv[5];
  job.o.visits = (uint32_t*)dv[6];
  const bool dyn = c->tree[1].n > 0;
  size_t smem = (size_t)maxlevel * (dyn ? 3 : 2) * qbc::kThreads * sizeof(uint32_t);
  int64_t blocks = (n + qbc::kThreads - 1) / qbc::kThreads;
  if (blocks > INT32_MAX) return fail(QBC_E_ARG, "qbc_trace_rays: too many rays");
  const bool exact = qbc::cube_shift_exact(probe);
  if (exact && dyn)
    qbc::rays_kernel<true, true><<<(unsigned)blocks, qbc::kThreads, smem, c->stream>>>(device_scene(c), job);
  else if (exact)
    qbc::rays_kernel<true, false><<<(unsigned)blocks, qbc::kThreads, smem, c->stream>>>(device_scene(c), job);
  else if (dyn)
    qbc::rays_kernel<false, true><<<(unsigned)blocks, qbc::kThreads, smem, c->stream>>>(device_scene(c), job);
  else
    qbc::rays_kernel<false, false><<<(unsigned)blocks, qbc::kThreads, smem, c->stream>>>(device_scene(c), job);
  QBC_CUDA(cudaGetLastError());
  ++c->launches;
  if (!on_device) {
    for (int k = 0; k < 7; ++k)
      if (*hs[k]) QBC_CUDA(cudaMemcpyAsync(*hs[k], dv[k], (size_t)n * bytes[k], cudaMemcpyDeviceToHost, c->stream));
    QBC_CUDA(cudaStreamSynchronize(c->stream));
  }
  return QBC_OK;
}

// ---------------------------------------------------------------------------
// Render without allocating (qbc_render_views_noalloc)
// ---------------------------------------------------------------------------

// Work-queue counters of qbc_render_views_noalloc: one per launch of 32
// views. File-scope static device memory, so the call needs no allocation;
// every GPU that loads the library holds these 256 bytes until exit.
static __device__ __align__(256) unsigned int qbc_noalloc_queues[QBC_NOALLOC_MAX_LAUNCHES];

namespace {

constexpr int kNoallocMaxDevices = 64;
std::mutex g_noalloc_mu;
unsigned int* g_noalloc_ptr[kNoallocMaxDevices] = {};

// Device address of the counters on the current device, looked up once per
// device (cudaGetSymbolAddress with that device current).
int noalloc_queues(int device, unsigned int** out) {
  if (device < 0 || device >= kNoallocMaxDevices)
    return fail(QBC_E_ARG, "qbc_render_views_noalloc: device %d beyond %d", device, kNoallocMaxDevices);
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[device]) {
    void* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, qbc_noalloc_queues);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(qbc_noalloc_queues)");
    g_noalloc_ptr[device] = static_cast<unsigned int*>(ptr);
  }
  *out = g_noalloc_ptr[device];
  return QBC_OK;
}

template <bool EXACT, bool DYN>
int launch_render_noalloc(qbc_ctx* c, const qbc::Batch& b, size_t smem, unsigned int* queue) {
  auto kern = qbc::render_kernel<EXACT, DYN, qbc::kFused, false>;
  QBC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024));
  int per_sm = 0;
  QBC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, qbc::kThreads, smem));
  if (per_sm < 1) return fail(QBC_E_STATE, "render_kernel: no block fits on an SM with %zu B shared memory", smem);
  if (c->blocks_per_sm > 0) per_sm = std::min(per_sm, c->blocks_per_sm);
  int64_t blocks = std::min<int64_t>((int64_t)per_sm * c->sm_count, ((int64_t)b.tiles_total + 3) / 4);
  blocks = std::max<int64_t>(blocks, 1);
  kern<<<(unsigned)blocks, qbc::kThreads, smem, c->stream>>>(device_scene(c), b, queue, qbc::Wave{});
  QBC_CUDA(cudaGetLastError());
  ++c->launches;
  return QBC_OK;
}

}  // namespace

extern "C" int qbc_render_views_noalloc(qbc_ctx* c, const qbc_view* views, const qbc_outputs* outs, int n) {
  qbc::clear_error();
  if (!c || (n > 0 && (!views || !outs))) return fail(QBC_E_ARG, "qbc_render_views_noalloc: null argument");
  if (n < 0) return fail(QBC_E_ARG, "qbc_render_views_noalloc: negative view count");
  if (n > QBC_NOALLOC_MAX_VIEWS)
    return fail(QBC_E_ARG, "qbc_render_views_noalloc: %d views exceed the maximum of %d per call (%d work-queue counters of 32 views)",
                n, QBC_NOALLOC_MAX_VIEWS, QBC_NOALLOC_MAX_LAUNCHES);
  if (n == 0) return QBC_OK;
  QBC_CUDA(cudaSetDevice(c->device));
  for (int i = 0; i < n; ++i) {
    int rc = check_view(views[i], i);
    if (rc) return rc;
    const qbc_outputs& o = outs[i];
    const void* ptrs[6] = {o.rgba8, o.rgba32f, o.flags, o.leaf, o.isp, o.visits};
    for (int k = 0; k < 6; ++k) {
      if (!ptrs[k]) continue;
      cudaPointerAttributes attr;
      cudaError_t e = cudaPointerGetAttributes(&attr, ptrs[k]);
      if (e != cudaSuccess || attr.type != cudaMemoryTypeDevice || attr.device != c->device) {
        cudaGetLastError();
        return fail(QBC_E_ARG, "qbc_render_views_noalloc: output %d of view %d is not device memory of device %d", k,
                    i, c->device);
      }
    }
  }
  unsigned int* queues = nullptr;
  int rc = noalloc_queues(c->device, &queues);
  if (rc) return rc;
  const int launches = (n + qbc::kMaxViewsPerLaunch - 1) / qbc::kMaxViewsPerLaunch;
  // the counters keep the previous call's values: start every used one at 0
  QBC_CUDA(cudaMemsetAsync(queues, 0, sizeof(unsigned int) * (size_t)launches, c->stream));
  const bool dyn = c->tree[1].n > 0;
  qbc::Batch b;  // on the stack: no host allocation either
  for (int l = 0; l < launches; ++l) {
    const int a = l * qbc::kMaxViewsPerLaunch;
    const int m = std::min(qbc::kMaxViewsPerLaunch, n - a);
    std::memset(&b, 0, sizeof(b));
    int tiles = 0, maxlevel = 0;
    bool exact = true;
    for (int i = 0; i < m; ++i) {
      qbc::ViewJob& J = b.job[i];
      J.v = views[a + i];
      J.o = outs[a + i];
      const int tw = 1 << c->tile_shift, th = 32 >> c->tile_shift;
      J.tiles_x = (views[a + i].width_px + tw - 1) / tw;
      J.tile_begin = tiles;
      tiles += J.tiles_x * ((views[a + i].height_px + th - 1) / th);
      maxlevel = std::max(maxlevel, views[a + i].maxlevel);
      exact = exact && qbc::cube_shift_exact(views[a + i]);
    }
    b.n = m;
    b.tiles_total = tiles;
    b.max_level = maxlevel;
    b.service_min = c->service_min;
    b.tile_shift = c->tile_shift;
    const size_t smem = ((size_t)(dyn ? 3 : 2) * maxlevel + qbc::kPixWords) * qbc::kThreads * sizeof(uint32_t);
    unsigned int* q = queues + l;
    if (exact)
      rc = dyn ? launch_render_noalloc<true, true>(c, b, smem, q) : launch_render_noalloc<true, false>(c, b, smem, q);
    else
      rc = dyn ? launch_render_noalloc<false, true>(c, b, smem, q) : launch_render_noalloc<false, false>(c, b, smem, q);
    if (rc) return rc;
  }
  return QBC_OK;
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
    collect_kernel<<<launch_grid(c, queued), 256, 0, c->stream>>>(*b, w, c->ds_x, c->ds_t, c->ds_kind,
                                                                  c->ds_count, c->ds_cap);
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

extern "C" int qbc_render(qbc_ctx* c, float width, float height, const float position[3], const float angle[3],
                          float lighta, int quality, int maxlevel, float basesize, int shoot, uint8_t* rgba8_out) {
  qbc::clear_error();
  if (!c || !rgba8_out) return fail(QBC_E_ARG, "qbc_render: null argument");
  qbc_view v;
  int rc = qbc_view_setup(width, height, position, angle, lighta, quality, maxlevel, basesize, shoot, 0.0f, &v);
  if (rc) return rc;
  qbc_outputs o;
  std::memset(&o, 0, sizeof(o));
  o.rgba8 = rgba8_out;
  return qbc_render_views(c, &v, &o, 1, 0);
}
