// The context behind a qbc_ctx handle and the helpers the library's
// translation units share (qbcuda.cu: context, uploads, builds, rendering;
// frame.cu: frame graphs and the autotuner; proposal.cu: the occluder
// network). Private to libqbcuda.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <vector>

#include "mlp.h"
#include "qbc_internal.h"
#include "qbcuda.h"
#include "render.cuh"

using qbc::fail;

struct DevTreeBuf {
  int4* child = nullptr;
  int32_t* model = nullptr;
  int64_t n = 0;    // node count of the array last uploaded
  int64_t cap = 0;  // nodes allocated
  // children's leaf boxes for pruning (boxes.cu), rebuilt lazily after a change
  uint32_t* cbox = nullptr;
  int64_t cbox_cap = 0;  // nodes
  int box_depth = -1;
  bool box_valid = false;
  // a GPU build leaves the exact node count on the device (d_count) and n at
  // the build's bound; the count is read back only when the host asks
  bool count_on_device = false;
  int32_t* d_count = nullptr;
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
  uint64_t attr_done = 0;  // kernel variants whose shared-memory limit is set (bit per variant)
  int service_min = qbc::kServiceMinDefault;
  int tile_shift = 3;     // 8x4 warp tiles
  int blocks_per_sm = 0;  // render blocks per SM (0: as many as fit)
  int proposal_gate = 500;  // per mille: minimum predicted occlusion probability to try a proposal
  int proposal_count = 3;   // network proposals tried per pixel (earliest first)
  int proposal_level = 8;   // level of the proposed cells when a render's options leave it 0
  int box_prune = 1;        // skip subtrees whose leaf boxes the ray misses
  int persistent = 1;       // fused frames on the persistent kernel (0: one thread per pixel)
  int split_trees = 0;      // two-tree fused frames as a one-tree and a two-tree launch
  int64_t launches = 0;
  qbc::BuildScratch build;       // GPU tree build scratch, kept for per-frame rebuilds
  void* build_input = nullptr;   // device copy of host build input
  int64_t build_input_cap = 0;   // bytes
  unsigned* derr = nullptr;      // device: qbc::DeviceError bits of kernels' input checks
  cudaStream_t copy = nullptr;   // host-output copies, overlapped with the next views' render
  std::vector<cudaEvent_t> copy_ev;  // one per chunk of a host-output render
  int32_t* counts = nullptr;     // device: node counts of GPU-built trees (one per tree)
};

// Node count of a tree; a GPU-built tree's count is read from the device
// (synchronizes).
int tree_count(qbc_ctx* c, int tree, int64_t* n);
// Report and clear the device-side input faults recorded since the last
// check (synchronizes).
int check_device_errors(qbc_ctx* c);
// Enqueue a per-frame dynamic update (skin, rebuild, normals); no allocation
// once the buffers have the update's size, no host synchronisation.
int dynamic_update(qbc_ctx* c, const qbc_dynamic_update* u);

constexpr size_t kStageMax = size_t(256) << 20;

inline int cuda_fail(cudaError_t e, const char* what) {
  return fail(QBC_E_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define QBC_CUDA(call)                            \
  do {                                            \
    cudaError_t e_ = (call);                      \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
  } while (0)

inline int ensure_stage(qbc_ctx* c, size_t bytes) {
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
inline int grow(T** p, int64_t* cap, int64_t need, size_t elem_bytes, const char* what) {
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

inline int launch_grid(const qbc_ctx* c, int64_t n) {
  int64_t blocks = (n + 255) / 256;
  int64_t maxb = (int64_t)std::max(c->sm_count, 1) * 16;
  return (int)std::max<int64_t>(1, std::min(blocks, maxb));
}

inline qbc::DevScene device_scene(const qbc_ctx* c) {
  qbc::DevScene s;
  s.box_words = nullptr;
  for (int t = 0; t < 2; ++t) {
    s.tree[t].child = c->tree[t].child;
    s.tree[t].model = c->tree[t].model;
    s.tree[t].n = (int32_t)c->tree[t].n;
    const bool boxes = c->box_prune && c->tree[t].box_valid && c->tree[t].box_depth >= 0;
    s.tree[t].cbox = boxes ? c->tree[t].cbox : nullptr;
    s.tree[t].box_depth = boxes ? c->tree[t].box_depth : 0;
    s.model[t].col = c->model[t].col;
    s.model[t].nrm = c->model[t].nrm;
    // the colour and normal arrays are separate uploads; a point index is
    // valid when both hold it
    s.model[t].n = (int32_t)std::min(c->model[t].n_col, c->model[t].n_nrm);
  }
  return s;
}

// Rebuild the leaf boxes of trees changed since the last build (allocates).
int ensure_boxes(qbc_ctx* c);

// Shared entry points of the translation units.
int check_view(const qbc_view& v, int i);
int check_render_opts(const qbc_render_opts* opts, int n);
int render_views_impl(qbc_ctx* c, const qbc_view* views, const qbc_outputs* outs, int n, int outputs_on_device,
                      const qbc_render_opts* opts, qbc_render_stats* stats);
// Proposals of every queued record of a two-pass render from the network
// (proposal.cu); the queue length is read on the device.
int propose_mlp(qbc_ctx* c, const qbc::Batch& b, const qbc::Wave& w);
// The context is going: free the graph's CUDA objects (frame.cu).
void detach_graph(qbc_graph* g);
