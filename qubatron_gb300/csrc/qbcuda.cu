// libqbcuda: context, uploads and the render kernel behind include/qbcuda.h.
//
// The render kernel is the per-pixel body of the reference's fragment shader
// src/qubatron/shaders/octree_fsh.c:399-464 (ray generation, primary ray,
// shadow ray, shading, light flare); the traversal is in trace.cuh. Build
// flags: -fmad=false -prec-div=true -prec-sqrt=true -ftz=false.

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <vector>

#include "qbc_internal.h"
#include "qbcuda.h"
#include "trace.cuh"

using qbc::fail;

namespace qbc {

constexpr int kThreads = 128;      // 4 warps; each warp shades an 8x4 pixel tile
constexpr int kTileW = 16;         // a block shades a 16x8 tile
constexpr int kTileH = 8;
constexpr int kMaxViewsPerLaunch = 32;

struct ViewJob {
  qbc_view v;
  qbc_outputs o;  // device pointers
  int32_t tiles_x;
  int32_t tile_begin;
  int32_t exact;  // cube recovery by inversion (see cube_shift_exact)
  int32_t pad;
};

struct Batch {
  ViewJob job[kMaxViewsPerLaunch];
  int32_t n;
  int32_t tiles_total;
};

// ---- main() helpers (octree_fsh.c:381-395 and GLSL built-ins) ----
__device__ __forceinline__ float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

__device__ __forceinline__ float3 normalize3(float3 v) {
  float len = sqrtf(dot3(v, v));
  return make_float3(v.x / len, v.y / len, v.z / len);
}

__device__ __forceinline__ float glsl_max(float x, float y) { return x < y ? y : x; }

__device__ __forceinline__ float3 quat_rotate(const float* q, float3 v) {
  // v + 2.0 * cross(q.xyz, cross(q.xyz, v) + q.w * v)
  float c1x = q[1] * v.z - q[2] * v.y;
  float c1y = q[2] * v.x - q[0] * v.z;
  float c1z = q[0] * v.y - q[1] * v.x;
  float ax = c1x + q[3] * v.x;
  float ay = c1y + q[3] * v.y;
  float az = c1z + q[3] * v.z;
  float c2x = q[1] * az - q[2] * ay;
  float c2y = q[2] * ax - q[0] * az;
  float c2z = q[0] * ay - q[1] * ax;
  return make_float3(v.x + 2.0f * c2x, v.y + 2.0f * c2y, v.z + 2.0f * c2z);
}

// GL float -> unorm8 for the RGBA8 colour target.
__device__ __forceinline__ uint32_t unorm8(float f) {
  if (!(f > 0.0f)) return 0u;
  if (f >= 1.0f) return 255u;
  return (uint32_t)(f * 255.0f + 0.5f);
}

template <bool EXACT>
__device__ __forceinline__ void shade_pixel(const DevScene& sc, const ViewJob& J, int i, int j, const Stack& st) {
  const qbc_view& v = J.v;
  const float4 bc = make_float4(v.basecube[0], v.basecube[1], v.basecube[2], v.basecube[3]);
  const float3 camfp = make_float3(v.camfp[0], v.camfp[1], v.camfp[2]);
  const float3 light = make_float3(v.light[0], v.light[1], v.light[2]);
  uint32_t f = 0;
  int32_t leaf[4] = {-1, -1, -1, -1};
  uint32_t vis[4] = {0, 0, 0, 0};
  float4 ispo = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  float4 col = ispo;
  bool written = true;

  // ray generation (octree_fsh.c:402-413); coord is the pixel centre
  float cx = ((float)i + 0.5f) * v.coord_scale[0];
  float cy = ((float)j + 0.5f) * v.coord_scale[1];
  float3 csv = make_float3(cx - v.cfp[0], cy - v.cfp[1], 0.0f - v.cfp[2]);
  csv = quat_rotate(v.qz, csv);
  csv = quat_rotate(v.qx, csv);

  float3 ncsv = normalize3(csv);
  float cosang = dot3(make_float3(v.ncamlight[0], v.ncamlight[1], v.ncamlight[2]), ncsv);
  bool flare = cosang > v.flare_cos && cosang <= 1.0f;

  TraceOut res;
  trace<EXACT>(sc, bc, v.maxlevel, camfp, csv, st, res);
  vis[0] = res.vis_s;
  vis[1] = res.vis_d;
  if (res.oob) f |= QBC_PX_OOB;
  if (res.status == kDiscard) {
    f |= QBC_PX_DISCARD;
    written = false;
  } else {
    if (res.status == kLeaf) {
      f |= QBC_PX_PRIMARY_LEAF;
      leaf[0] = res.leaf_s;
      leaf[1] = res.leaf_d;
    }
    ispo = res.isp;
    col = res.col;

    if (res.isp.w > 0.0f) {
      // shadow ray and shading (octree_fsh.c:431-449)
      f |= QBC_PX_SHADED;
      float3 lghtv = make_float3(res.isp.x - light.x, res.isp.y - light.y, res.isp.z - light.z);
      TraceOut lc;
      trace<EXACT>(sc, bc, v.maxlevel, light, lghtv, st, lc);
      vis[2] = lc.vis_s;
      vis[3] = lc.vis_d;
      if (lc.oob) f |= QBC_PX_OOB;
      if (lc.status == kDiscard) {
        f |= QBC_PX_DISCARD;
        written = false;
      } else {
        if (lc.status == kLeaf) {
          f |= QBC_PX_SHADOW_LEAF;
          leaf[2] = lc.leaf_s;
          leaf[3] = lc.leaf_d;
        }
        float ix = lc.isp.x - res.isp.x, iy = lc.isp.y - res.isp.y, iz = lc.isp.z - res.isp.z;
        float sqr = ix * ix + iy * iy + iz * iz;
        float3 nl = normalize3(make_float3(-lghtv.x, -lghtv.y, -lghtv.z));
        float3 nn = normalize3(make_float3(res.nrm.x, res.nrm.y, res.nrm.z));
        float3 nc = normalize3(make_float3(-csv.x, -csv.y, -csv.z));
        float lght_nrm_ang = glsl_max(dot3(nl, nn), 0.0f);
        float camv_nrm_ang = glsl_max(dot3(nc, nn), 0.0f);
        float lit = (15.0f < sqr) ? 0.0f : 1.0f;  // step(sqr, 15.0)
        if (lit != 0.0f) f |= QBC_PX_LIT;
        float k = 0.1f + 0.2f * camv_nrm_ang + lght_nrm_ang * lit * 0.7f;
        col.x = col.x * k;
        col.y = col.y * k;
        col.z = col.z * k;
        col.z *= 0.7f;
        float g = (float)v.shoot * camv_nrm_ang * 0.1f;
        col.x += g;
        col.y += g;
        col.z += g;
      }
    }

    if (written && flare) {
      // light flare (octree_fsh.c:452-459)
      f |= QBC_PX_FLARE_TEST;
      float3 lghtv = make_float3(light.x - camfp.x, light.y - camfp.y, light.z - camfp.z);
      TraceOut lc;
      trace<EXACT>(sc, bc, v.maxlevel, camfp, lghtv, st, lc);
      if (lc.oob) f |= QBC_PX_OOB;
      if (lc.status == kDiscard) {
        f |= QBC_PX_DISCARD;
        written = false;
      } else {
        float resv_x = lc.isp.x - camfp.x;
        if (resv_x / lghtv.x > 1.0f) {
          f |= QBC_PX_FLARE_WHITE;
          col = make_float4(1.0f, 1.0f, 1.0f, 1.0f);
        }
      }
    }
  }
  if (!written) col = make_float4(0.0f, 0.0f, 0.0f, 0.0f);

  const int64_t o = (int64_t)j * v.width_px + i;
  const qbc_outputs& out = J.o;
  if (out.rgba8)
    reinterpret_cast<uint32_t*>(out.rgba8)[o] =
        unorm8(col.x) | (unorm8(col.y) << 8) | (unorm8(col.z) << 16) | (unorm8(col.w) << 24);
  if (out.rgba32f) reinterpret_cast<float4*>(out.rgba32f)[o] = col;
  if (out.flags) out.flags[o] = f;
  if (out.leaf) reinterpret_cast<int4*>(out.leaf)[o] = make_int4(leaf[0], leaf[1], leaf[2], leaf[3]);
  if (out.isp) reinterpret_cast<float4*>(out.isp)[o] = ispo;
  if (out.visits) reinterpret_cast<uint4*>(out.visits)[o] = make_uint4(vis[0], vis[1], vis[2], vis[3]);
}

__global__ void __launch_bounds__(kThreads) render_kernel(DevScene sc, const __grid_constant__ Batch batch) {
  extern __shared__ uint32_t smem[];
  const int tile = blockIdx.x;
  // the view owning this tile: last job with tile_begin <= tile
  int lo = 0, hi = batch.n - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (batch.job[mid].tile_begin <= tile)
      lo = mid;
    else
      hi = mid - 1;
  }
  const ViewJob& J = batch.job[lo];
  const int t = tile - J.tile_begin;
  const int tx = t % J.tiles_x, ty = t / J.tiles_x;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int px = tx * kTileW + (warp & 1) * 8 + (lane & 7);
  const int py = ty * kTileH + (warp >> 1) * 4 + (lane >> 3);
  if (px >= J.v.width_px || py >= J.v.height_px) return;
  Stack st{smem + threadIdx.x, kThreads};
  if (J.exact)
    shade_pixel<true>(sc, J, px, py, st);
  else
    shade_pixel<false>(sc, J, px, py, st);
}

struct RayJob {
  const float* pos;
  const float* dir;
  int64_t n;
  float4 bc;
  int32_t maxlevel;
  int32_t exact;
  qbc_ray_hits o;
};

template <bool EXACT>
__device__ __forceinline__ void ray_query(const DevScene& sc, const RayJob& J, int64_t i, const Stack& st) {
  float3 p = make_float3(J.pos[3 * i], J.pos[3 * i + 1], J.pos[3 * i + 2]);
  float3 d = make_float3(J.dir[3 * i], J.dir[3 * i + 1], J.dir[3 * i + 2]);
  TraceOut r;
  trace<EXACT>(sc, J.bc, J.maxlevel, p, d, st, r);
  if (J.o.status) J.o.status[i] = r.status;
  if (J.o.leaf) reinterpret_cast<int2*>(J.o.leaf)[i] = make_int2(r.leaf_s, r.leaf_d);
  if (J.o.model) reinterpret_cast<int2*>(J.o.model)[i] = make_int2(r.model_s, r.model_d);
  if (J.o.isp) reinterpret_cast<float4*>(J.o.isp)[i] = r.isp;
  if (J.o.col) reinterpret_cast<float4*>(J.o.col)[i] = r.col;
  if (J.o.nrm) reinterpret_cast<float4*>(J.o.nrm)[i] = r.nrm;
  if (J.o.visits) reinterpret_cast<uint2*>(J.o.visits)[i] = make_uint2(r.vis_s, r.vis_d);
}

__global__ void __launch_bounds__(kThreads) rays_kernel(DevScene sc, const __grid_constant__ RayJob job) {
  extern __shared__ uint32_t smem[];
  const int64_t i = blockIdx.x * (int64_t)kThreads + threadIdx.x;
  if (i >= job.n) return;
  Stack st{smem + threadIdx.x, kThreads};
  if (job.exact)
    ray_query<true>(sc, job, i, st);
  else
    ray_query<false>(sc, job, i, st);
}

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
    s.tree[t].n = c->tree[t].n;
    s.model[t].col = c->model[t].col;
    s.model[t].nrm = c->model[t].nrm;
    // the colour and normal arrays are separate uploads; a point index is
    // valid when both hold it
    s.model[t].n = std::min(c->model[t].n_col, c->model[t].n_nrm);
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
  c->stream = c->own;
  *out = c;
  return QBC_OK;
}

extern "C" int qbc_destroy(qbc_ctx* c) {
  if (!c) return QBC_OK;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  for (int t = 0; t < 2; ++t) {
    cudaFree(c->tree[t].child);
    cudaFree(c->tree[t].model);
    cudaFree(c->model[t].col);
    cudaFree(c->model[t].nrm);
  }
  cudaFree(c->stage);
  cudaFree(c->scratch);
  if (c->own) cudaStreamDestroy(c->own);
  delete c;
  return QBC_OK;
}

extern "C" int qbc_set_stream(qbc_ctx* c, void* stream) {
  if (!c) return fail(QBC_E_ARG, "qbc_set_stream: null context");
  c->stream = stream ? (cudaStream_t)stream : c->own;
  return QBC_OK;
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

extern "C" int qbc_upload(qbc_ctx* c, const void* data, int type, size_t size, size_t itemsize, size_t start,
                          size_t end, int buftype) {
  qbc::clear_error();
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
    if (hi > lo) {
      int rc = ensure_stage(c, (size_t)std::min(hi - lo, chunk) * node_bytes);
      if (rc) return rc;
    }
    for (int64_t a = lo; a < hi; a += chunk) {
      int64_t b = std::min(hi, a + chunk);
      QBC_CUDA(cudaMemcpyAsync(c->stage, base + a * node_bytes, (size_t)(b - a) * node_bytes, cudaMemcpyHostToDevice,
                               c->stream));
      qbc::repack_nodes_kernel<<<launch_grid(c, b - a), 256, 0, c->stream>>>(
          (const int4*)c->stage, b - a, t.child + 2 * a, t.model + a);
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
    if (hi > lo) {
      int rc = ensure_stage(c, (size_t)std::min(hi - lo, chunk) * 12);
      if (rc) return rc;
    }
    for (int64_t a = lo; a < hi; a += chunk) {
      int64_t b = std::min(hi, a + chunk);
      QBC_CUDA(cudaMemcpyAsync(c->stage, base + a * 12, (size_t)(b - a) * 12, cudaMemcpyHostToDevice, c->stream));
      qbc::expand_attr_kernel<<<launch_grid(c, b - a), 256, 0, c->stream>>>((const float*)c->stage, b - a,
                                                                             *arr + a, 1.0f);
      QBC_CUDA(cudaGetLastError());
      ++c->launches;
    }
  }
  QBC_CUDA(cudaStreamSynchronize(c->stream));
  return QBC_OK;
}

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

int launch_batch(qbc_ctx* c, const qbc_view* views, const qbc_outputs* dev_outs, int n) {
  qbc::Batch* b = new qbc::Batch();
  int tiles = 0, maxlevel = 0;
  for (int i = 0; i < n; ++i) {
    qbc::ViewJob& J = b->job[i];
    J.v = views[i];
    J.o = dev_outs[i];
    J.tiles_x = (views[i].width_px + qbc::kTileW - 1) / qbc::kTileW;
    int tiles_y = (views[i].height_px + qbc::kTileH - 1) / qbc::kTileH;
    J.tile_begin = tiles;
    J.exact = qbc::cube_shift_exact(views[i]) ? 1 : 0;
    tiles += J.tiles_x * tiles_y;
    maxlevel = std::max(maxlevel, views[i].maxlevel);
  }
  b->n = n;
  b->tiles_total = tiles;
  size_t smem = (size_t)maxlevel * 3 * qbc::kThreads * sizeof(uint32_t);
  static bool attr_set = false;
  if (!attr_set) {
    cudaFuncSetAttribute(qbc::render_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 1024);
    attr_set = true;
  }
  qbc::render_kernel<<<tiles, qbc::kThreads, smem, c->stream>>>(device_scene(c), *b);
  delete b;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "render_kernel launch");
  ++c->launches;
  return QBC_OK;
}

}  // namespace

extern "C" int qbc_render_views(qbc_ctx* c, const qbc_view* views, const qbc_outputs* outs, int n,
                                int outputs_on_device) {
  qbc::clear_error();
  if (!c || (n > 0 && (!views || !outs))) return fail(QBC_E_ARG, "qbc_render_views: null argument");
  if (n < 0) return fail(QBC_E_ARG, "qbc_render_views: negative view count");
  QBC_CUDA(cudaSetDevice(c->device));
  for (int i = 0; i < n; ++i) {
    int rc = check_view(views[i], i);
    if (rc) return rc;
  }

  if (outputs_on_device) {
    for (int a = 0; a < n; a += qbc::kMaxViewsPerLaunch) {
      int rc = launch_batch(c, views + a, outs + a, std::min(qbc::kMaxViewsPerLaunch, n - a));
      if (rc) return rc;
    }
    return QBC_OK;
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
    int rc = launch_batch(c, views + a, dev.data() + a, std::min(qbc::kMaxViewsPerLaunch, n - a));
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
  job.exact = qbc::cube_shift_exact(probe) ? 1 : 0;
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
  size_t smem = (size_t)maxlevel * 3 * qbc::kThreads * sizeof(uint32_t);
  int64_t blocks = (n + qbc::kThreads - 1) / qbc::kThreads;
  if (blocks > INT32_MAX) return fail(QBC_E_ARG, "qbc_trace_rays: too many rays");
  qbc::rays_kernel<<<(unsigned)blocks, qbc::kThreads, smem, c->stream>>>(device_scene(c), job);
  QBC_CUDA(cudaGetLastError());
  ++c->launches;
  if (!on_device) {
    for (int k = 0; k < 7; ++k)
      if (*hs[k]) QBC_CUDA(cudaMemcpyAsync(*hs[k], dv[k], (size_t)n * bytes[k], cudaMemcpyDeviceToHost, c->stream));
    QBC_CUDA(cudaStreamSynchronize(c->stream));
  }
  return QBC_OK;
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
