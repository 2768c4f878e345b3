// Frame graphs (qbc_graph_*) and the autotuner (qbc_autotune) of libqbcuda:
// both drive whole frames through render_views_impl on a context's stream.

#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <initializer_list>
#include <memory>
#include <vector>

#include "qbc_ctx.h"

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
  int32_t persistent;
  int32_t proposal_level;
  int32_t split_trees;
};

bool same_signature(const FrameSignature& a, const FrameSignature& b) {
  for (int t = 0; t < 2; ++t) {
    const qbc::DevTree &ta = a.scene.tree[t], &tb = b.scene.tree[t];
    const qbc::DevModel &ma = a.scene.model[t], &mb = b.scene.model[t];
    if (ta.child != tb.child || ta.model != tb.model || ta.n != tb.n) return false;
    if (ta.cbox != tb.cbox || ta.box_depth != tb.box_depth) return false;
    if (ma.col != mb.col || ma.nrm != mb.nrm || ma.n != mb.n) return false;
  }
  return a.rec == b.rec && a.rec_cap == b.rec_cap && a.pixlog == b.pixlog && a.pixlog_cap == b.pixlog_cap &&
         a.net_w == b.net_w && a.net_b == b.net_b && a.stream == b.stream && a.service_min == b.service_min &&
         a.proposal_gate == b.proposal_gate && a.tile_shift == b.tile_shift && a.blocks_per_sm == b.blocks_per_sm &&
         a.proposal_count == b.proposal_count && a.persistent == b.persistent &&
         a.proposal_level == b.proposal_level && a.split_trees == b.split_trees;
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
  f.persistent = c->persistent;
  f.proposal_level = c->proposal_level;
  f.split_trees = c->split_trees;
  return f;
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
  qbc_dynamic_update update;  // captured in front of the render when has_update
  bool has_update = false;
};

namespace {

int capture_frame(qbc_graph* g, const qbc_view* views, cudaGraph_t* out) {
  qbc_ctx* c = g->ctx;
  QBC_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  int rc = g->has_update ? dynamic_update(c, &g->update) : QBC_OK;
  if (!rc) rc = render_views_impl(c, views, g->outs.data(), g->n, 1, g->has_opts ? &g->opts : nullptr, nullptr);
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

namespace {

int capture_impl(qbc_ctx* c, const qbc_dynamic_update* update, const qbc_view* views, const qbc_outputs* dev_outs,
                 int n, const qbc_render_opts* opts, qbc_graph** out) {
  if (!c || !views || !dev_outs || !out || n <= 0) return fail(QBC_E_ARG, "qbc_graph_capture: bad argument");
  int rc = check_render_opts(opts, n);
  if (rc) return rc;
  QBC_CUDA(cudaSetDevice(c->device));
  // one eager frame first: buffers grown and kernel attributes set before
  // the capture, which must not allocate
  if (update) rc = dynamic_update(c, update);
  if (!rc) rc = render_views_impl(c, views, dev_outs, n, 1, opts, nullptr);
  if (rc) return rc;
  QBC_CUDA(cudaStreamSynchronize(c->stream));
  std::unique_ptr<qbc_graph> g(new qbc_graph());
  if (update) {
    g->update = *update;
    g->has_update = true;
  }
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

}  // namespace

extern "C" int qbc_graph_capture(qbc_ctx* c, const qbc_view* views, const qbc_outputs* dev_outs, int n,
                                 const qbc_render_opts* opts, qbc_graph** out) {
  qbc::clear_error();
  return capture_impl(c, nullptr, views, dev_outs, n, opts, out);
}

extern "C" int qbc_graph_capture_dynamic(qbc_ctx* c, const qbc_dynamic_update* update, const qbc_view* views,
                                         const qbc_outputs* dev_outs, int n, const qbc_render_opts* opts,
                                         qbc_graph** out) {
  qbc::clear_error();
  if (!update) return fail(QBC_E_ARG, "qbc_graph_capture_dynamic: null update");
  return capture_impl(c, update, views, dev_outs, n, opts, out);
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
  // leaf boxes rebuilt outside the capture (that allocates and synchronises)
  int brc = ensure_boxes(c);
  if (brc) return brc;
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

// A tuning setting: warp tile, blocks per SM, service threshold, for frames
// with network proposals the gate (1000: off), count and cell level, and for
// fused frames with two trees whether they split.
struct TuneSetting {
  int shift, blocks, service;
  int gate, count, level;
  int split;
};

TuneSetting current_setting(const qbc_ctx* c) {
  return {c->tile_shift, c->blocks_per_sm, c->service_min, c->proposal_gate, c->proposal_count, c->proposal_level,
          c->split_trees};
}

void apply_setting(qbc_ctx* c, const TuneSetting& s) {
  c->tile_shift = s.shift;
  c->blocks_per_sm = s.blocks;
  c->service_min = s.service;
  c->proposal_gate = s.gate;
  c->proposal_count = s.count;
  c->proposal_level = s.level;
  c->split_trees = s.split;
}

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
  float best_ms = 0.0f;
  int rc = time_frames(c, views, outs, n, opts, reps, ev, &best_ms);
  if (rc) return rc;
  res->ms_initial = best_ms;
  res->candidates = 1;
  auto consider = [&](const TuneSetting& s) -> int {
    apply_setting(c, s);
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
  // each option swept with the others at their best so far
  auto vary = [&](int TuneSetting::*f, std::initializer_list<int> vals) -> int {
    for (int v : vals) {
      if (v == best->*f) continue;
      TuneSetting s = *best;
      s.*f = v;
      const int e = consider(s);
      if (e) return e;
    }
    return QBC_OK;
  };
  // network proposals first: whether they pay at all (gate 1000 is off),
  // how confident the network must be, how many to try, at which level
  if (opts && opts->proposals == QBC_PROPOSE_MLP) {
    if ((rc = vary(&TuneSetting::gate, {1000, 900, 700, 500, 300, 0}))) return rc;
    if (best->gate < 1000) {
      if ((rc = vary(&TuneSetting::count, {1, 2, 3}))) return rc;
      if (opts->proposal_level == 0 && (rc = vary(&TuneSetting::level, {5, 6, 7, 8}))) return rc;
    }
  }
  // then the schedule, one option at a time
  if ((rc = vary(&TuneSetting::service, {1, 2, 3, 4, 6, 8, 12, 16}))) return rc;
  if ((rc = vary(&TuneSetting::shift, {1, 2, 3, 4, 5}))) return rc;
  // (5 blocks of a two-tree kernel fit a 164 KB shared-memory carveout:
  // more L1 for fewer warps)
  if ((rc = vary(&TuneSetting::blocks, {0, 2, 3, 4, 5, 6, 8}))) return rc;
  // a fused frame with two trees: one launch or the split, at the schedule
  // found (its second launch's tail weighs differently per schedule)
  if ((!opts || !opts->two_pass) && c->persistent && c->tree[1].n > 0 &&
      (rc = vary(&TuneSetting::split, {0, 1})))
    return rc;
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
  const TuneSetting initial = current_setting(c);
  TuneSetting best = initial;
  rc = autotune_impl(c, views, dev_outs, n, opts, reps, ev, &best, result);
  const TuneSetting keep = rc ? initial : best;
  apply_setting(c, keep);
  cudaEventDestroy(ev[0]);
  cudaEventDestroy(ev[1]);
  if (rc) return rc;
  result->tile_width = 1 << keep.shift;
  result->blocks_per_sm = keep.blocks;
  result->service_min = keep.service;
  result->proposal_gate = keep.gate;
  result->proposal_count = keep.count;
  result->proposal_level = keep.level;
  result->split_trees = keep.split;
  return QBC_OK;
}
