// libqbcuda: context, uploads, tree builds and edits, and the render kernels
// behind include/qbcuda.h (frame graphs and the autotuner are in frame.cu,
// the occluder network in proposal.cu).
//
// The kernels are in render.cuh (per-pixel shader body, persistent) and
// walker.cuh (the traversal). Build flags: -fmad=false -prec-div=true
// -prec-sqrt=true -ftz=false.

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <memory>
#include <new>
#include <vector>

#include "qbc_ctx.h"

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
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->copy, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&c->derr, sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMemset(c->derr, 0, sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMalloc(&c->counts, 2 * sizeof(int32_t));
  if (e != cudaSuccess) {
    if (c->copy) cudaStreamDestroy(c->copy);
    if (c->own) cudaStreamDestroy(c->own);
    delete c;
    return cuda_fail(e, "qbc_create");
  }
  c->stream = c->own;
  c->net.err = c->derr;
  c->tree[0].d_count = c->counts;
  c->tree[1].d_count = c->counts + 1;
  *out = c;
  return QBC_OK;
}

extern "C" int qbc_destroy(qbc_ctx* c) {
  if (!c) return QBC_OK;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  for (qbc_graph* g : c->graphs) detach_graph(g);
  for (int t = 0; t < 2; ++t) {
    cudaFree(c->tree[t].child);
    cudaFree(c->tree[t].model);
    cudaFree(c->tree[t].cbox);
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
  for (cudaEvent_t ev : c->copy_ev) cudaEventDestroy(ev);
  if (c->copy) cudaStreamDestroy(c->copy);
  qbc::build_release(&c->build);
  cudaFree(c->build_input);
  cudaFree(c->derr);
  cudaFree(c->counts);
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
    if (value < 0 || value > 1000) return fail(QBC_E_ARG, "qbc_set_option: proposal gate %d outside 0..1000", value);
    c->proposal_gate = value;
    return QBC_OK;
  }
  if (option == QBC_OPT_PROPOSAL_LEVEL) {
    if (value < 1 || value > QBC_MAX_LEVEL)
      return fail(QBC_E_ARG, "qbc_set_option: proposal level %d outside 1..%d", value, QBC_MAX_LEVEL);
    c->proposal_level = value;
    return QBC_OK;
  }
  if (option == QBC_OPT_PROPOSAL_COUNT) {
    if (value < 1 || value > 3) return fail(QBC_E_ARG, "qbc_set_option: proposal count %d outside 1..3", value);
    c->proposal_count = value;
    return QBC_OK;
  }
  if (option == QBC_OPT_BOX_PRUNE) {
    if (value < 0 || value > 1) return fail(QBC_E_ARG, "qbc_set_option: box pruning %d (0 or 1)", value);
    c->box_prune = value;
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
  if (option == QBC_OPT_PERSISTENT) {
    if (value < 0 || value > 1) return fail(QBC_E_ARG, "qbc_set_option: persistent %d (0 or 1)", value);
    c->persistent = value;
    return QBC_OK;
  }
  if (option == QBC_OPT_SPLIT_TREES) {
    if (value < 0 || value > 1) return fail(QBC_E_ARG, "qbc_set_option: split trees %d (0 or 1)", value);
    c->split_trees = value;
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
  if (option == QBC_OPT_PROPOSAL_LEVEL) {
    *value = c->proposal_level;
    return QBC_OK;
  }
  if (option == QBC_OPT_BOX_PRUNE) {
    *value = c->box_prune;
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
  if (option == QBC_OPT_PERSISTENT) {
    *value = c->persistent;
    return QBC_OK;
  }
  if (option == QBC_OPT_SPLIT_TREES) {
    *value = c->split_trees;
    return QBC_OK;
  }
  return fail(QBC_E_ARG, "qbc_get_option: unknown option %d", option);
}

int check_device_errors(qbc_ctx* c) {
  unsigned h = 0;
  QBC_CUDA(cudaMemcpyAsync(&h, c->derr, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  QBC_CUDA(cudaStreamSynchronize(c->stream));
  if (!h) return QBC_OK;
  QBC_CUDA(cudaMemsetAsync(c->derr, 0, sizeof(unsigned), c->stream));
  QBC_CUDA(cudaStreamSynchronize(c->stream));
  if (h & qbc::kErrRecordOverflow)
    return fail(QBC_E_STATE, "render: the record queue of a split frame was full; some pixels were not written");
  if (h & qbc::kErrMmaTimeout)
    return fail(QBC_E_TIMEOUT, "proposal network: a tensor-core wait gave up; the proposals of that render are incomplete");
  if (h & qbc::kErrSkinBone) return fail(QBC_E_ARG, "qbc_skin_rigid: a bone index was outside the bone set (point skinned with bone 0)");
  if (h & qbc::kErrBuildPoint)
    return fail(QBC_E_ARG, "tree build: a point was negative, too large or not finite (left out of the tree)");
  return fail(QBC_E_ARG, "tree build: an octet was outside 0..7 (its path left out of the tree)");
}

int tree_count(qbc_ctx* c, int tree, int64_t* n) {
  DevTreeBuf& tb = c->tree[tree];
  if (tb.count_on_device) {
    int32_t h = 0;
    QBC_CUDA(cudaMemcpyAsync(&h, tb.d_count, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
    QBC_CUDA(cudaStreamSynchronize(c->stream));
    *n = h;
  } else {
    *n = tb.n;
  }
  return QBC_OK;
}

extern "C" int qbc_synchronize(qbc_ctx* c) {
  qbc::clear_error();
  if (!c) return fail(QBC_E_ARG, "qbc_synchronize: null context");
  QBC_CUDA(cudaSetDevice(c->device));
  QBC_CUDA(cudaStreamSynchronize(c->stream));
  return check_device_errors(c);
}

extern "C" int qbc_tree_nodes(qbc_ctx* c, int tree, int64_t* n) {
  qbc::clear_error();
  if (!c || !n || tree < 0 || tree > 1) return fail(QBC_E_ARG, "qbc_tree_nodes: bad argument");
  QBC_CUDA(cudaSetDevice(c->device));
  int rc = tree_count(c, tree, n);
  if (rc) return rc;
  return check_device_errors(c);
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
    t.count_on_device = false;
    t.box_valid = false;  // leaf boxes rebuilt before the next render
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
  // a host array may be reused once the call returns; a device source is
  // read in stream order
  if (!device_src) QBC_CUDA(cudaStreamSynchronize(c->stream));
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
                                  float* __restrict__ on, unsigned* __restrict__ bad) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    int b = bone[i];
    if (b < 0 || b >= n_bones) {
      atomicOr(bad, qbc::kErrSkinBone);
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

// The same with the bone set read from device memory when the kernel runs
// (a captured frame then sees the bones written before each replay).
__global__ void skin_rigid_dev_kernel(const float* __restrict__ rp, const float* __restrict__ rn,
                                      const int32_t* __restrict__ bone, int64_t n, int n_bones,
                                      const float* __restrict__ bones, float* __restrict__ op,
                                      float* __restrict__ on, unsigned* __restrict__ bad) {
  __shared__ float m_all[QBC_MAX_BONES * 12];
  for (int k = threadIdx.x; k < n_bones * 12; k += blockDim.x) m_all[k] = bones[k];
  __syncthreads();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    int b = bone[i];
    if (b < 0 || b >= n_bones) {
      atomicOr(bad, qbc::kErrSkinBone);
      b = 0;
    }
    const float* m = m_all + 12 * b;
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
  skin_rigid_kernel<<<launch_grid(c, n), 256, 0, c->stream>>>(rest_pnts, rest_nrms, bone, n, n_bones, bs, out_pnts,
                                                              out_nrms, c->derr);
  QBC_CUDA(cudaGetLastError());
  ++c->launches;
  return QBC_OK;
}

// ---------------------------------------------------------------------------
// GPU tree build (octree_insert_point / octree_insert_path order)
// ---------------------------------------------------------------------------

namespace {

// Host build input is checked here (so a bad point fails the call at once)
// and copied to the device.
int stage_build_input(qbc_ctx* c, const float* pnts, const int32_t* octets, int64_t n, int levels,
                      const void** dev) {
  if (pnts) {
    for (int64_t i = 0; i < 3 * n; ++i)
      if (!(pnts[i] >= 0.0f && pnts[i] < 1.0e30f))
        return fail(QBC_E_ARG, "tree build: point %lld is negative, too large or not finite", (long long)(i / 3));
  } else {
    for (int64_t i = 0; i < n * levels; ++i)
      if (octets[i] < 0 || octets[i] > 7)
        return fail(QBC_E_ARG, "tree build: octet %d of path %lld is outside 0..7", octets[i], (long long)(i / levels));
  }
  const size_t bytes = pnts ? (size_t)n * 12 : (size_t)n * levels * 4;
  if (c->build_input_cap < (int64_t)bytes) {
    int rc = grow(reinterpret_cast<char**>(&c->build_input), &c->build_input_cap, (int64_t)bytes, 1, "tree build input");
    if (rc) return rc;
  }
  QBC_CUDA(cudaMemcpyAsync(c->build_input, pnts ? (const void*)pnts : (const void*)octets, bytes,
                           cudaMemcpyHostToDevice, c->stream));
  *dev = c->build_input;
  return QBC_OK;
}

// A GPU build into tree `tree` (qbc_build_tree, qbc_build_tree_paths,
// qbc_load_flat). Buffers are sized for the build's node bound, so a build of
// the same size as the last one allocates nothing, and nothing is read back:
// the exact node count stays on the device. A static-tree build frees the
// build scratch afterwards (a one-time build); a dynamic-tree build keeps it
// for the next frame.
int build_into(qbc_ctx* c, int tree, const float* pnts, const int32_t* octets, int64_t n, float basesize, int levels,
               int64_t first_index, int on_device) {
  if (!c || tree < 0 || tree > 1) return fail(QBC_E_ARG, "tree build: bad context or tree id");
  if (n < 0 || (n > 0 && !pnts && !octets)) return fail(QBC_E_ARG, "tree build: bad input");
  if (pnts && !(basesize > 0.0f)) return fail(QBC_E_ARG, "tree build: basesize must be positive");
  if (levels < 0 || levels > 21) return fail(QBC_E_ARG, "tree build: levels %d outside 0..21", levels);
  QBC_CUDA(cudaSetDevice(c->device));
  const void* dev = pnts ? (const void*)pnts : (const void*)octets;
  if (!on_device && n > 0) {
    int rc = stage_build_input(c, pnts, octets, n, levels, &dev);
    if (rc) return rc;
  }
  int rc = qbc::build_reserve(&c->build, n, levels);
  if (rc) return rc;
  DevTreeBuf& tb = c->tree[tree];
  const int64_t bound = qbc::build_node_bound(n, levels);
  if (tb.cap < bound || !tb.child) {
    int64_t cap = 0;
    rc = grow(&tb.child, &cap, bound, 32, "octree child blocks");
    if (!rc) rc = grow(&tb.model, &tb.cap, bound, 4, "octree model indices");
    if (rc) return rc;
  }
  if (tb.cbox_cap < bound || !tb.cbox) {
    rc = grow(&tb.cbox, &tb.cbox_cap, bound, 64, "octree leaf boxes");
    if (rc) return rc;
  }
  rc = qbc::build_tree_async(pnts ? static_cast<const float*>(dev) : nullptr,
                             pnts ? nullptr : static_cast<const int32_t*>(dev), n, basesize, levels, first_index,
                             &c->build, reinterpret_cast<int32_t*>(tb.child), tb.model, tb.cbox, tb.d_count, c->derr,
                             c->stream, c->sm_count * 8, &c->launches);
  if (rc) return rc;
  tb.n = bound;
  tb.count_on_device = true;
  tb.box_depth = levels <= QBC_MAX_LEVEL ? levels : -1;
  tb.box_valid = true;
  if (tree == 0) {
    // a one-time build: the exact count bounds the kernels' index checks
    int64_t exact = 0;
    rc = tree_count(c, 0, &exact);
    if (rc) return rc;
    tb.n = exact;
    tb.count_on_device = false;
    qbc::build_release(&c->build);
    cudaFree(c->build_input);
    c->build_input = nullptr;
    c->build_input_cap = 0;
  }
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

int dynamic_update(qbc_ctx* c, const qbc_dynamic_update* u) {
  if (!c || !u) return fail(QBC_E_ARG, "qbc_dynamic_update: null argument");
  if (u->n < 0 || (u->n > 0 && (!u->rest_pnts || !u->bone || !u->bones || !u->pnts)))
    return fail(QBC_E_ARG, "qbc_dynamic_update: null array");
  if (u->n_bones < 1 || u->n_bones > QBC_MAX_BONES)
    return fail(QBC_E_ARG, "qbc_dynamic_update: %d bones outside 1..%d", u->n_bones, QBC_MAX_BONES);
  if ((u->rest_nrms == nullptr) != (u->nrms == nullptr))
    return fail(QBC_E_ARG, "qbc_dynamic_update: give both normal arrays or neither");
  if (u->n > INT32_MAX) return fail(QBC_E_ARG, "qbc_dynamic_update: %lld points exceed int32 indices", (long long)u->n);
  QBC_CUDA(cudaSetDevice(c->device));
  if (u->n > 0) {
    skin_rigid_dev_kernel<<<launch_grid(c, u->n), 256, 0, c->stream>>>(u->rest_pnts, u->rest_nrms, u->bone, u->n,
                                                                         u->n_bones, u->bones, u->pnts, u->nrms,
                                                                         c->derr);
    QBC_CUDA(cudaGetLastError());
    ++c->launches;
  }
  int64_t n = u->n;
  const float* pts = u->n > 0 ? u->pnts : reinterpret_cast<const float*>(&n);
  int rc = build_into(c, 1, pts, nullptr, u->n, u->basesize, u->levels, 0, 1);
  if (rc) return rc;
  if (u->nrms && u->n > 0) {
    const size_t bytes = (size_t)u->n * 12;
    rc = upload_impl(c, u->nrms, QBC_GL_FLOAT, bytes, 12, 0, bytes, QBC_DYNAMIC_NORMAL, true);
  }
  return rc;
}

extern "C" int qbc_dynamic_update_run(qbc_ctx* c, const qbc_dynamic_update* u) {
  qbc::clear_error();
  return dynamic_update(c, u);
}


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
  if (nodes) {
    int rc2 = tree_count(c, tree, nodes);
    if (rc2) return rc2;
  }
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
  QBC_CUDA(cudaSetDevice(c->device));
  int64_t n = 0;
  int rc0 = tree_count(c, tree, &n);
  if (!rc0) rc0 = check_device_errors(c);
  if (rc0) return rc0;
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

int ensure_boxes(qbc_ctx* c) {
  if (!c->box_prune) return QBC_OK;
  for (int t = 0; t < 2; ++t) {
    DevTreeBuf& tb = c->tree[t];
    if (tb.box_valid) continue;
    tb.box_depth = -1;
    if (tb.n > 0) {
      if (tb.cbox_cap < tb.n) {
        int rc = grow(&tb.cbox, &tb.cbox_cap, tb.cap > tb.n ? tb.cap : tb.n, 64, "octree leaf boxes");
        if (rc) return rc;
      }
      QBC_CUDA(cudaMemsetAsync(tb.cbox, 0, (size_t)tb.n * 64, c->stream));
      int depth = -1;
      int rc = qbc::build_child_boxes(reinterpret_cast<const int32_t*>(tb.child), tb.n, tb.cbox, c->stream, &depth,
                                      &c->launches);
      if (rc) return rc;
      tb.box_depth = depth;
    }
    tb.box_valid = true;
  }
  return QBC_OK;
}

// ---------------------------------------------------------------------------
// Render
// ---------------------------------------------------------------------------

namespace qbc {

// Proposals for the records of a two-pass render: the t of the first leaf a
// previous plain walk of the same pixel logged (when it shadowed), or seeded
// pseudo-random t values (exactness tests exercise the proposal path with
// both).
__global__ void fill_logged_proposals(const __grid_constant__ Batch batch, const __grid_constant__ Wave wave) {
  const unsigned total = min(*wave.qcount, wave.cap);
  for (unsigned q = blockIdx.x * blockDim.x + threadIdx.x; q < total; q += gridDim.x * blockDim.x) {
    uint32_t* r = wave.rec + (size_t)q * kRecWords;
    const ViewJob& J = batch.job[r[kRecView] & 0xFFu];
    const uint32_t xy = r[kRecXY];
    const float t = wave.pixlog[J.pixel_begin + (int64_t)(xy >> 16) * J.v.width_px + (xy & 0xFFFFu)];
    reinterpret_cast<float&>(r[kRecProp]) = t;
    reinterpret_cast<float&>(r[kRecProp + 1]) = -1.0f;
    reinterpret_cast<float&>(r[kRecProp + 2]) = -1.0f;
  }
}

__global__ void fill_random_proposals(const __grid_constant__ Wave wave, unsigned long long seed) {
  const unsigned total = min(*wave.qcount, wave.cap);
  for (unsigned q = blockIdx.x * blockDim.x + threadIdx.x; q < total; q += gridDim.x * blockDim.x) {
    uint32_t* r = wave.rec + (size_t)q * kRecWords;
    unsigned long long z = seed + 0x9E3779B97F4A7C15ull * (r[kRecXY] + 0x10001ull * (r[kRecView] & 0xFFu) + 1);
    for (int k = 0; k < 3; ++k) {
      z += 0x9E3779B97F4A7C15ull;
      unsigned long long x = z;
      x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
      x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
      x ^= x >> 31;
      reinterpret_cast<float&>(r[kRecProp + k]) = (float)(x >> 40) * (1.0f / 16777216.0f);
    }
  }
}

}  // namespace qbc

int check_view(const qbc_view& v, int i) {
  if (v.width_px < 1 || v.height_px < 1 || v.width_px > 65536 || v.height_px > 65536)
    return fail(QBC_E_ARG, "view %d: %dx%d pixels outside 1..65536", i, v.width_px, v.height_px);
  if (v.maxlevel < 0 || v.maxlevel > QBC_MAX_LEVEL)
    return fail(QBC_E_ARG, "view %d: maxlevel %d outside 0..%d", i, v.maxlevel, QBC_MAX_LEVEL);
  return QBC_OK;
}

namespace {

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


// Statistics of the last render: the shade passes' counters of a two-pass
// render, the leaf-box words of an instrumented one (synchronizes).
int read_stats(qbc_ctx* c, qbc_render_stats* stats, bool two) {
  if (!stats) return QBC_OK;
  unsigned long long h[qbc::kStatCount];
  unsigned int q[2] = {0u, 0u};
  QBC_CUDA(cudaMemcpyAsync(h, c->wstats, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  if (two) QBC_CUDA(cudaMemcpyAsync(q, c->wcount, sizeof(q), cudaMemcpyDeviceToHost, c->stream));
  QBC_CUDA(cudaStreamSynchronize(c->stream));
  stats->queued = two ? q[0] : h[qbc::kStatSplitQueued];
  stats->shadow_rays = h[qbc::kStatShadowRays];
  stats->shadow_visits = h[qbc::kStatShadowVisits];
  stats->proposals_tried = h[qbc::kStatPropTried];
  stats->proposals_proven = h[qbc::kStatPropProven];
  stats->proposal_visits = h[qbc::kStatPropVisits];
  stats->box_words = h[qbc::kStatBoxWords];
  return QBC_OK;
}

template <bool EXACT, bool DYN, int MODE, bool PROP>
int launch_render(qbc_ctx* c, const qbc::Batch& b, size_t smem, const qbc::Wave& wave) {
  auto kern = qbc::render_kernel<EXACT, DYN, MODE, PROP>;
  const int variant = (EXACT ? 1 : 0) + (DYN ? 2 : 0) + 4 * MODE + (PROP ? 16 : 0);
  if (!(c->attr_done & (1ull << variant))) {
    QBC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024));
    c->attr_done |= 1ull << variant;
  }
  int per_sm = 0;
  QBC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, qbc::kThreads, smem));
  if (per_sm < 1) return fail(QBC_E_STATE, "render_kernel: no block fits on an SM with %zu B shared memory", smem);
  if (MODE == qbc::kFused && !PROP) c->render_blocks[(EXACT ? 1 : 0) + (DYN ? 2 : 0)] = per_sm;
  if (c->blocks_per_sm > 0) per_sm = std::min(per_sm, c->blocks_per_sm);
  // persistent: one wave of resident blocks, never more blocks than warp tiles
  int64_t blocks = (int64_t)per_sm * c->sm_count;
  // (the split frame's two-tree kernel takes records, then the tiles its
  // one-tree kernel left: the tile counter carries over)
  constexpr bool tiles_only = MODE == qbc::kFused || MODE == qbc::kPrimaryPass || MODE == qbc::kSplitStatic;
  if (tiles_only) blocks = std::min<int64_t>(blocks, ((int64_t)b.tiles_total + 3) / 4);
  blocks = std::max<int64_t>(blocks, 1);
  if (tiles_only) QBC_CUDA(cudaMemsetAsync(c->queue, 0, sizeof(unsigned int), c->stream));
  qbc::DevScene sc = device_scene(c);
  for (int i = 0; i < b.n; ++i)
    if (b.job[i].o.visits) sc.box_words = c->wstats + qbc::kStatBoxWords;  // an instrumented render
  kern<<<(unsigned)blocks, qbc::kThreads, smem, c->stream>>>(sc, b, c->queue, wave);
  QBC_CUDA(cudaGetLastError());
  ++c->launches;
  return QBC_OK;
}

// The plain schedule: one warp per 32-pixel tile, 4 tiles per block.
template <bool EXACT, bool DYN>
int launch_simple(qbc_ctx* c, const qbc::Batch& b, size_t smem) {
  auto kern = qbc::simple_kernel<EXACT, DYN>;
  const int variant = 32 + (EXACT ? 1 : 0) + (DYN ? 2 : 0);
  if (!(c->attr_done & (1ull << variant))) {
    QBC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024));
    c->attr_done |= 1ull << variant;
  }
  const int64_t blocks = std::max<int64_t>(1, ((int64_t)b.tiles_total + 3) / 4);
  qbc::DevScene sc = device_scene(c);
  for (int i = 0; i < b.n; ++i)
    if (b.job[i].o.visits) sc.box_words = c->wstats + qbc::kStatBoxWords;
  kern<<<(unsigned)blocks, qbc::kThreads, smem, c->stream>>>(sc, b);
  QBC_CUDA(cudaGetLastError());
  ++c->launches;
  return QBC_OK;
}

// A fused two-tree frame in two launches: the one-tree kernel walks every ray
// that provably leaves the dynamic tree alone and queues each pixel whose
// next ray may not (with its state and the phase to resume at); the
// two-tree kernel finishes the queued pixels, then the tiles the one-tree
// kernel left. A pixel leaves the one-tree kernel at most once. The queue
// holds a quarter of the batch's pixels (kSplitRecWords words each, two
// record units of the context's buffer); once it may not hold every pixel
// in flight (at most 64 per warp after a warp's last look at the count: the
// 32 in its lanes and a new tile's 32), the one-tree kernel takes no new
// tile.
template <bool EXACT, bool DYN>
int launch_split(qbc_ctx* c, const qbc::Batch& b, size_t smem, int64_t pixels) {
  if constexpr (EXACT && DYN) {
    const int64_t reserve = (int64_t)64 * 4 * 32 * c->sm_count;  // 64 per warp, 32 blocks of 4 warps per SM at most
    const int64_t want = std::min<int64_t>(std::max<int64_t>(pixels / 4, 2 * reserve), pixels + reserve);
    // (the record buffer counts kRecWords units; a split record takes two)
    constexpr int64_t kUnits = qbc::kSplitRecWords / qbc::kRecWords;
    if (c->rec_cap < kUnits * want) {
      int rc = grow(&c->rec, &c->rec_cap, kUnits * want, (size_t)qbc::kRecWords * 4, "render records");
      if (rc) return rc;
    }
    const int64_t split_cap = c->rec_cap / kUnits;
    qbc::Wave w{};
    w.rec = c->rec;
    w.qcount = c->wcount;
    w.qnext = c->wcount + 1;
    w.stats = c->wstats;
    w.cap = (uint32_t)std::min<int64_t>(split_cap, 0xFFFFFFFFll);
    w.stop = (split_cap >= pixels && pixels <= 0xFFFFFFFFll) ? 0xFFFFFFFFu : (uint32_t)(w.cap - reserve);
    w.err = c->derr;
    QBC_CUDA(cudaMemsetAsync(c->wcount, 0, 2 * sizeof(unsigned int), c->stream));
    const size_t smem1 = qbc::render_smem(b.max_level, false, false);
    int rc = launch_render<true, false, qbc::kSplitStatic, false>(c, b, smem1, w);
    if (rc) return rc;
    return launch_render<true, true, qbc::kSplitFinish, false>(c, b, smem, w);
  } else {
    (void)b;
    (void)smem;
    (void)pixels;
    return fail(QBC_E_STATE, "split frame: needs exact cubes and two trees");
  }
}

// Whether a fused frame runs split: two trees, exact cubes, the dynamic
// tree's leaf boxes built below its root and reached by the batch's depth.
bool split_frame(const qbc_ctx* c, const qbc::Batch& b, bool exact, bool dyn) {
  if (!exact || !dyn || !c->persistent || !c->split_trees) return false;
  const qbc::DevTree t = device_scene(c).tree[1];
  return t.cbox != nullptr && t.box_depth > 1 && b.max_level >= t.box_depth;
}

template <bool EXACT, bool DYN>
int launch_modes(qbc_ctx* c, const qbc::Batch& b, size_t smem, const qbc_render_opts* opts, int64_t pixels) {
  if ((!opts || !opts->two_pass) && !c->persistent) return launch_simple<EXACT, DYN>(c, b, smem);
  if ((!opts || !opts->two_pass) && split_frame(c, b, EXACT, DYN)) return launch_split<EXACT, DYN>(c, b, smem, pixels);
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
  // a gate of 1000 switches the network's proposals off: no inference, the
  // plain shade pass
  const bool mlp_off = opts->proposals == QBC_PROPOSE_MLP && c->proposal_gate >= 1000;
  w.nprop = (opts->proposals != QBC_PROPOSE_NONE && !mlp_off) ? 3 : 0;
  w.pdepth = opts->proposal_level > 0 ? opts->proposal_level : c->proposal_level;
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
  } else if (opts->proposals == QBC_PROPOSE_MLP && !mlp_off) {
    rc = propose_mlp(c, b, w);
    if (rc) return rc;
  }
  if (w.nprop > 0) rc = launch_render<EXACT, DYN, qbc::kShadePass, true>(c, b, qbc::render_smem(b.max_level, DYN, true), w);
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
  const size_t smem = qbc::render_smem(maxlevel, dyn, false);
  int rc;
  if (exact)
    rc = dyn ? launch_modes<true, true>(c, *b, smem, opts, pixels) : launch_modes<true, false>(c, *b, smem, opts, pixels);
  else
    rc = dyn ? launch_modes<false, true>(c, *b, smem, opts, pixels) : launch_modes<false, false>(c, *b, smem, opts, pixels);
  delete b;
  return rc;
}

}  // namespace

int check_render_opts(const qbc_render_opts* opts, int n) {
  if (opts && (opts->proposals < QBC_PROPOSE_NONE || opts->proposals > QBC_PROPOSE_RANDOM))
    return fail(QBC_E_ARG, "qbc_render_views_ex: unknown proposal source %d", opts->proposals);
  if (opts && opts->proposals != QBC_PROPOSE_NONE && !opts->two_pass)
    return fail(QBC_E_ARG, "qbc_render_views_ex: proposals need two_pass");
  if (opts && (opts->proposal_level < 0 || opts->proposal_level > QBC_MAX_LEVEL))
    return fail(QBC_E_ARG, "qbc_render_views_ex: proposal_level %d outside 0..%d", opts->proposal_level, QBC_MAX_LEVEL);
  // the render log indexes pixels within one launch of kMaxViewsPerLaunch
  // views; other two-pass renders run batch after batch
  if (opts && opts->two_pass && (opts->log || opts->proposals == QBC_PROPOSE_LOGGED) && n > qbc::kMaxViewsPerLaunch)
    return fail(QBC_E_ARG, "qbc_render_views_ex: logged two-pass renders take at most %d views per call",
                qbc::kMaxViewsPerLaunch);
  return QBC_OK;
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

int render_views_impl(qbc_ctx* c, const qbc_view* views, const qbc_outputs* outs, int n, int outputs_on_device,
                      const qbc_render_opts* opts, qbc_render_stats* stats) {
  if (!c || (n > 0 && (!views || !outs))) return fail(QBC_E_ARG, "qbc_render_views: null argument");
  if (n < 0) return fail(QBC_E_ARG, "qbc_render_views: negative view count");
  QBC_CUDA(cudaSetDevice(c->device));
  for (int i = 0; i < n; ++i) {
    int rc = check_view(views[i], i);
    if (rc) return rc;
  }

  int brc = ensure_boxes(c);
  if (brc) return brc;
  const bool two = opts && opts->two_pass;
  if (two || stats) QBC_CUDA(cudaMemsetAsync(c->wstats, 0, qbc::kStatCount * sizeof(unsigned long long), c->stream));
  if (outputs_on_device) {
    for (int a = 0; a < n; a += qbc::kMaxViewsPerLaunch) {
      int rc = launch_batch(c, views + a, outs + a, std::min(qbc::kMaxViewsPerLaunch, n - a), opts);
      if (rc) return rc;
    }
    return read_stats(c, stats, two);
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
  // Views in chunks of about a quarter of the pixels (at least 16M pixels,
  // at most one launch's views): a chunk's copies to the host run on the
  // copy stream while the next chunk renders. Each extra launch costs a
  // tail, so small frames stay whole (16 x 1080p: 2 chunks; 32 x 4K: 4). A
  // logged render stays one launch (its log indexes the pixels of one
  // launch).
  int64_t total_px = 0;
  for (int i = 0; i < n; ++i) total_px += (int64_t)views[i].width_px * views[i].height_px;
  const bool logged = opts && (opts->log || opts->proposals == QBC_PROPOSE_LOGGED);
  const int64_t target = logged ? INT64_MAX : std::max<int64_t>(total_px / 4, int64_t(16) << 20);
  int chunk = 0;
  for (int a = 0; a < n;) {
    int m = 0;
    int64_t px_chunk = 0;
    while (a + m < n && m < qbc::kMaxViewsPerLaunch && (m == 0 || px_chunk < target)) {
      px_chunk += (int64_t)views[a + m].width_px * views[a + m].height_px;
      ++m;
    }
    int rc = launch_batch(c, views + a, dev.data() + a, m, opts);
    if (rc) return rc;
    if ((int)c->copy_ev.size() <= chunk) {
      cudaEvent_t ev = nullptr;
      QBC_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
      c->copy_ev.push_back(ev);
    }
    QBC_CUDA(cudaEventRecord(c->copy_ev[(size_t)chunk], c->stream));
    QBC_CUDA(cudaStreamWaitEvent(c->copy, c->copy_ev[(size_t)chunk], 0));
    for (int i = a; i < a + m; ++i) {
      size_t px = (size_t)views[i].width_px * views[i].height_px;
      qbc_outputs h = outs[i];
      for (int k = 0; k < 6; ++k) {
        void* dst = *out_slot(h, k);
        if (!dst) continue;
        QBC_CUDA(cudaMemcpyAsync(dst, *out_slot(dev[i], k), px * kOutBytes[k], cudaMemcpyDeviceToHost, c->copy));
      }
    }
    a += m;
    ++chunk;
  }
  QBC_CUDA(cudaStreamSynchronize(c->copy));
  QBC_CUDA(cudaStreamSynchronize(c->stream));
  return read_stats(c, stats, two);
}

// Ray queries: one wave of resident blocks (lanes take rays by grid stride),
// never more blocks than the rays need.
template <bool EXACT, bool DYN>
int launch_rays(qbc_ctx* c, const qbc::RayJob& job, size_t smem) {
  auto kern = qbc::rays_kernel<EXACT, DYN>;
  int per_sm = 0;
  QBC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, qbc::kThreads, smem));
  if (per_sm < 1) return fail(QBC_E_STATE, "rays_kernel: no block fits on an SM with %zu B shared memory", smem);
  const int64_t blocks = std::max<int64_t>(
      1, std::min<int64_t>((int64_t)per_sm * c->sm_count, (job.n + qbc::kThreads - 1) / qbc::kThreads));
  kern<<<(unsigned)blocks, qbc::kThreads, smem, c->stream>>>(device_scene(c), job);
  QBC_CUDA(cudaGetLastError());
  ++c->launches;
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
  {
    int brc = ensure_boxes(c);
    if (brc) return brc;
  }
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
  job.service_min = c->service_min;
  const bool dyn = c->tree[1].n > 0;
  const size_t smem = (size_t)maxlevel * (dyn ? 3 : 2) * qbc::kThreads * sizeof(uint32_t);
  const bool exact = qbc::cube_shift_exact(probe);
  int rc = exact ? (dyn ? launch_rays<true, true>(c, job, smem) : launch_rays<true, false>(c, job, smem))
                 : (dyn ? launch_rays<false, true>(c, job, smem) : launch_rays<false, false>(c, job, smem));
  if (rc) return rc;
  if (!on_device) {
    for (int k = 0; k < 7; ++k)
      if (*hs[k]) QBC_CUDA(cudaMemcpyAsync(*hs[k], dv[k], (size_t)n * bytes[k], cudaMemcpyDeviceToHost, c->stream));
    QBC_CUDA(cudaStreamSynchronize(c->stream));
  }
  return QBC_OK;
}

namespace qbc {

// Camera rays of selected pixels of one view: (csv, cos of the angle to the
// light) per pixel, from the same camera_ray the render kernels call.
__global__ void camera_rays_kernel(const __grid_constant__ qbc_view v, const int32_t* px, const int32_t* py,
                                   int64_t n, float4* out) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
    out[k] = camera_ray(v, px[k], py[k]);
}

}  // namespace qbc

extern "C" int qbc_camera_rays(qbc_ctx* c, const qbc_view* view, const int32_t* px, const int32_t* py, int64_t n,
                               float* out, int on_device) {
  qbc::clear_error();
  if (!c || !view || (n > 0 && (!px || !py || !out))) return fail(QBC_E_ARG, "qbc_camera_rays: null argument");
  if (n < 0) return fail(QBC_E_ARG, "qbc_camera_rays: negative pixel count");
  int rc = check_view(*view, 0);
  if (rc) return rc;
  if (n == 0) return QBC_OK;
  QBC_CUDA(cudaSetDevice(c->device));
  const int32_t* dpx = px;
  const int32_t* dpy = py;
  float4* dout = reinterpret_cast<float4*>(out);
  if (!on_device) {
    // pixel indices and rays staged in the context's scratch
    const size_t idx = ((size_t)n * 4 + 255) & ~size_t(255);
    const size_t need = 2 * idx + (size_t)n * 16;
    if (need > c->scratch_bytes) {
      if (c->scratch) QBC_CUDA(cudaFree(c->scratch));
      c->scratch = nullptr;
      c->scratch_bytes = 0;
      cudaError_t e = cudaMalloc(&c->scratch, need);
      if (e != cudaSuccess) return fail(QBC_E_NOMEM, "camera-ray scratch of %zu bytes: %s", need, cudaGetErrorString(e));
      c->scratch_bytes = need;
    }
    char* base = (char*)c->scratch;
    QBC_CUDA(cudaMemcpyAsync(base, px, (size_t)n * 4, cudaMemcpyHostToDevice, c->stream));
    QBC_CUDA(cudaMemcpyAsync(base + idx, py, (size_t)n * 4, cudaMemcpyHostToDevice, c->stream));
    dpx = (const int32_t*)base;
    dpy = (const int32_t*)(base + idx);
    dout = (float4*)(base + 2 * idx);
  }
  qbc::camera_rays_kernel<<<launch_grid(c, n), 256, 0, c->stream>>>(*view, dpx, dpy, n, dout);
  QBC_CUDA(cudaGetLastError());
  ++c->launches;
  if (!on_device) {
    QBC_CUDA(cudaMemcpyAsync(out, dout, (size_t)n * 16, cudaMemcpyDeviceToHost, c->stream));
    QBC_CUDA(cudaStreamSynchronize(c->stream));
  }
  return QBC_OK;
}

// ---------------------------------------------------------------------------
// Render without allocating (qbc_render_views_noalloc)
// ---------------------------------------------------------------------------

// Work-queue counters of qbc_render_views_noalloc: one per launch of 32
// views. File-scope static device memory, so the call needs no allocation;
// every GPU that loads the library holds these 32 bytes until exit.
static __device__ __align__(256) unsigned int qbc_noalloc_queues[QBC_NOALLOC_MAX_LAUNCHES];
static_assert(QBC_NOALLOC_MAX_VIEWS <= QBC_NOALLOC_MAX_LAUNCHES * qbc::kMaxViewsPerLaunch,
              "every launch of a maximal no-allocation call needs its own counter");

namespace {

// Shared-memory limit of a fused render_kernel variant, set once per context
// (the same per-context cache launch_render uses). Setting it also loads the
// kernel's code under lazy module loading.
template <bool EXACT, bool DYN>
int fused_attr(qbc_ctx* c) {
  const int variant = (EXACT ? 1 : 0) + (DYN ? 2 : 0);
  if (!(c->attr_done & (1ull << variant))) {
    QBC_CUDA(cudaFuncSetAttribute(qbc::render_kernel<EXACT, DYN, qbc::kFused, false>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024));
    c->attr_done |= 1ull << variant;
  }
  return QBC_OK;
}

// Set-up of a no-allocation render on the context's device (current): the
// four fused kernel variants are loaded and given their shared-memory limit
// (on the context's first call; loading code can take device memory, so it
// happens here and not in a later frame), and the counters' device address
// is looked up with that device current. The lookup runs on every call, so
// an address never outlives the primary context it came from.
int noalloc_setup(qbc_ctx* c, unsigned int** out) {
  int rc = fused_attr<true, true>(c);
  if (!rc) rc = fused_attr<true, false>(c);
  if (!rc) rc = fused_attr<false, true>(c);
  if (!rc) rc = fused_attr<false, false>(c);
  if (rc) return rc;
  void* ptr = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&ptr, qbc_noalloc_queues);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(qbc_noalloc_queues)");
  *out = static_cast<unsigned int*>(ptr);
  return QBC_OK;
}

template <bool EXACT, bool DYN>
int launch_render_noalloc(qbc_ctx* c, const qbc::Batch& b, size_t smem, unsigned int* queue) {
  auto kern = qbc::render_kernel<EXACT, DYN, qbc::kFused, false>;
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
  int rc = noalloc_setup(c, &queues);
  if (rc) return rc;
  const int launches = (n + qbc::kMaxViewsPerLaunch - 1) / qbc::kMaxViewsPerLaunch;
  if (launches > QBC_NOALLOC_MAX_LAUNCHES)
    return fail(QBC_E_ARG, "qbc_render_views_noalloc: %d launches exceed the %d counters", launches,
                QBC_NOALLOC_MAX_LAUNCHES);
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
    const size_t smem = qbc::render_smem(maxlevel, dyn, false);
    unsigned int* q = queues + l;
    if (exact)
      rc = dyn ? launch_render_noalloc<true, true>(c, b, smem, q) : launch_render_noalloc<true, false>(c, b, smem, q);
    else
      rc = dyn ? launch_render_noalloc<false, true>(c, b, smem, q) : launch_render_noalloc<false, false>(c, b, smem, q);
    if (rc) return rc;
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
