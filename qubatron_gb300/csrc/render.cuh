// Render and ray-query kernels on the resumable walker (walker.cuh).
//
// render_kernel is the per-pixel body of the reference's fragment shader
// (src/qubatron/shaders/octree_fsh.c:399-464): ray generation, primary ray,
// shadow ray from the light, shading, light flare. It is persistent: every
// warp takes 32-pixel tiles (8x4 by default, QBC_OPT_TILE_WIDTH) from a
// global queue, and a lane whose ray ended
// continues at once with the next ray of its pixel (shadow, flare) or with
// the next pixel of its warp's tile, so lanes do not idle behind the
// slowest ray of the warp.
#pragma once

#include "qbc_internal.h"
#include "qbcuda.h"
#include "walker.cuh"

namespace qbc {

constexpr int kThreads = 128;  // 4 warps
constexpr int kMaxViewsPerLaunch = 32;
constexpr int kPixWords = 28;  // per-lane pixel state words in shared memory (at most)

struct ViewJob {
  qbc_view v;
  qbc_outputs o;  // device pointers
  int32_t tiles_x;      // warp tiles per row
  int32_t tile_begin;   // first global tile index of this view
  int64_t pixel_begin;  // first pixel index of this view within the batch
};

struct Batch {
  ViewJob job[kMaxViewsPerLaunch];
  int32_t n;
  int32_t tiles_total;
  int32_t max_level;    // largest maxlevel of the batch: stack depth
  int32_t service_min;  // lanes that must wait before a warp services them
  int32_t tile_shift;   // warp tile: 2^tile_shift x 32 / 2^tile_shift pixels
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

// Camera ray of pixel (i, j) of a view (octree_fsh.c:401-418): the screen
// vector ctp - cfp rotated by the yaw and pitch quaternions (csv), and the
// cosine of its angle to the light direction (the flare test's argument).
__device__ __forceinline__ float4 camera_ray(const qbc_view& v, int i, int j) {
  float cx = ((float)i + 0.5f) * v.coord_scale[0];
  float cy = ((float)j + 0.5f) * v.coord_scale[1];
  float3 csv = make_float3(cx - v.cfp[0], cy - v.cfp[1], 0.0f - v.cfp[2]);
  csv = quat_rotate(v.qz, csv);
  csv = quat_rotate(v.qx, csv);
  float3 ncsv = normalize3(csv);
  float cosang = dot3(make_float3(v.ncamlight[0], v.ncamlight[1], v.ncamlight[2]), ncsv);
  return make_float4(csv.x, csv.y, csv.z, cosang);
}

// The flare test acos(cosang) < 0.02 as a cosine threshold.
__device__ __forceinline__ bool flare_wanted(const qbc_view& v, float cosang) {
  return cosang > v.flare_cos && cosang <= 1.0f;
}

// GL float -> unorm8 for the RGBA8 colour target.
__device__ __forceinline__ uint32_t unorm8(float f) {
  if (!(f > 0.0f)) return 0u;
  if (f >= 1.0f) return 255u;
  return (uint32_t)(f * 255.0f + 0.5f);
}

__device__ __forceinline__ float4 view_bc(const qbc_view& v) {
  return make_float4(v.basecube[0], v.basecube[1], v.basecube[2], v.basecube[3]);
}

// The basecube as the kernels hold it: an EXACT launch has only views with
// basecube (+0, S, S, S) (cube_shift_exact), so one register holds it.
template <bool EXACT>
__device__ __forceinline__ float4 held_bc(const qbc_view& v) {
  const float s = v.basecube[3];
  return EXACT ? make_float4(0.0f, s, s, s) : view_bc(v);
}

// Per-lane pixel state in shared memory, word k at px[k * kThreads].
enum PixWord : int {
  kPxView = 0, kPxXY, kPxFlags,
  kPxCsv,                  // 3 words: camera ray direction
  kPxIsp = kPxCsv + 3,     // 4 words: primary intersection
  kPxCol = kPxIsp + 4,     // 4 words: colour (primary texel, then shaded)
  kPxNrm = kPxCol + 4,     // 3 words: primary normal
  kPxLeaf = kPxNrm + 3,    // 4 words: primary leaf s, d; shadow leaf s, d
  kPxVis = kPxLeaf + 4,    // 4 words: visits primary s, d; shadow s, d
  kPxProp = kPxVis + 4,    // 3 words: proposed shadow-ray t of the shade pass
  kPxEnd = kPxProp + 3
};
static_assert(kPxEnd <= kPixWords, "pixel state");
// Pixel state words the host allocates for a kernel: the kernels that test
// no proposals leave the proposal words out. Each word is 512 bytes of a
// 128-thread block; without them six blocks of the two-tree kernel fit a
// 196 KB shared-memory carveout instead of 228 KB, which doubles its L1
// cache (hit rate 33 % -> 63 %, 2-3 % less time); the one-tree kernels
// measured the same either way.
__host__ __device__ constexpr int pix_words(bool prop) { return prop ? kPxEnd : kPxProp; }

// Dynamic shared memory of a render kernel: its stack (2 words per level,
// 3 with two trees) and its pixel state, per thread of a block.
__host__ __device__ constexpr size_t render_smem(int max_level, bool dyn, bool prop) {
  return ((size_t)(dyn ? 3 : 2) * (size_t)max_level + (size_t)pix_words(prop)) * kThreads * sizeof(uint32_t);
}

// Records: 16 words per pixel one kernel hands to the next (the primary pass
// to the shade pass of a two-pass render; a split frame's one-tree kernel
// to its two-tree kernel). The camera ray, the primary texel and the normal
// are not carried: the reader recomputes them from the view, the pixel and
// the primary leaf, with the writer's own loads and arithmetic.
enum RecWord : int {
  kRecView = 0,              // view index (bits 0-7) | phase to resume at << 8 (split frames)
  kRecXY, kRecFlags,
  kRecIsp,                   // 4 words: primary intersection
  kRecLeaf = kRecIsp + 4,    // 2 words: primary leaf s, d
  kRecVis = kRecLeaf + 2,    // 2 words: primary visits s, d
  kRecProp = kRecVis + 2,    // 3 floats: proposals (two-pass; written between the passes)
  kRecShadow = kRecProp,     // split frames resuming at the flare ray: shadow leaf s, d, visits s, d
  kRecLogT = kRecProp + 3,   // float: t of the plain shadow walk's first leaf, -1 if none
  kRecLogLit,                // lit bit of the plain shadow walk
  kRecWords,
  // a split frame's records carry the state that a shade pass would
  // recompute: its two-tree kernel then resumes a pixel with no reloads
  // (its queue holds a quarter of the pixels, so they may be larger)
  kRecCsv = kRecWords,       // 3 words: camera ray direction
  kRecCol = kRecCsv + 3,     // 4 words: colour (primary texel, or shaded)
  kRecNrm = kRecCol + 4,     // 3 words: primary normal
  kSplitRecWords = 32
};
static_assert(kRecWords == 16 && kRecShadow + 4 <= kRecWords && kRecNrm + 3 <= kSplitRecWords, "record words");

enum Phase : int { kIdle = 0, kPrimary = 1, kShadow = 2, kFlare = 3, kProposal = 4 };
enum Mode : int { kFused = 0, kPrimaryPass = 1, kShadePass = 2, kSplitStatic = 3, kSplitFinish = 4 };

// Statistics of a render (uint64 each): the shade pass's counters, and the
// leaf-box words read by the walks of an instrumented render.
enum Stat : int {
  kStatShadowRays = 0,   // plain shadow walks
  kStatShadowVisits,     // node visits of plain shadow walks
  kStatPropTried,        // proposal walks
  kStatPropProven,       // shadow rays settled by a proposal
  kStatPropVisits,       // node visits of proposal walks
  kStatBoxWords,         // leaf-box words read (renders with a visits output)
  kStatSplitQueued,      // pixels a split frame's one-tree kernel handed on
  kStatCount = 8
};

struct Wave {
  uint32_t* rec;                // records (kRecWords words each; kSplitRecWords in a split frame)
  unsigned int* qcount;         // records written (by the primary pass, or a split frame's one-tree kernel)
  unsigned int* qnext;          // shade-pass work counter
  unsigned long long* stats;    // kStatCount counters
  uint32_t cap;                 // record capacity
  int32_t log;                  // shade pass: log the plain walk's first leaf
  int32_t nprop;                // proposals per record to try (0..3)
  int32_t pdepth;               // level of the proposed cells
  float* pixlog;                // per pixel of the batch: logged first-leaf t (-1 none), when log
  uint32_t stop;                // kSplitStatic: no new tile once qcount exceeds this
  unsigned* err;                // DeviceError bits (a split frame's record overflow)
};

// Internal flag: the pixel's camera ray is within the flare angle. The public
// QBC_PX_FLARE_TEST is set only when the flare ray is actually traced.
constexpr uint32_t kWantFlare = 1u << 31;

struct PixRef {
  uint32_t* base;
  __device__ __forceinline__ uint32_t& w(int k) const { return base[k * kThreads]; }
  __device__ __forceinline__ float& f(int k) const { return reinterpret_cast<float&>(base[k * kThreads]); }
};

// Lanes below this one in the warp (a special register: nothing held).
__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Octets of a point down to `depth` levels (octree.c:100-109), root first.
__device__ __forceinline__ uint32_t point_path(float3 q, float basesize, int depth) {
  uint32_t k = 0;
  float size = basesize;
  for (int level = 0; level < depth; ++level) {
    size /= 2.0f;
    int octet = (int)(q.x / size) % 2;
    int yi = (int)(q.y / size) % 2;
    int zi = (int)(q.z / size) % 2;
    if (yi == 0) octet += 2;
    if (zi == 0) octet += 4;
    k = (k << 3) | (uint32_t)octet;
  }
  return k;
}

// Record q of a pixel whose state words are px (stride kThreads), to resume
// at `phase` (0: a two-pass record, for the shade pass; else a split
// frame's, kSplitRecWords long). A pixel that resumes at its primary ray
// needs only its view and position.
__device__ __forceinline__ void write_record(uint32_t* r, const uint32_t* px, uint32_t phase) {
  r[kRecView] = px[kPxView * kThreads] | (phase << 8);
  r[kRecXY] = px[kPxXY * kThreads];
  if (phase == kPrimary) return;
  r[kRecFlags] = px[kPxFlags * kThreads];
#pragma unroll
  for (int k = 0; k < 4; ++k) r[kRecIsp + k] = px[(kPxIsp + k) * kThreads];
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    r[kRecLeaf + k] = px[(kPxLeaf + k) * kThreads];
    r[kRecVis + k] = px[(kPxVis + k) * kThreads];
  }
  if (phase == kFlare) {
    // the shadow walk already ran: its leaf and visits
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      r[kRecShadow + k] = px[(kPxLeaf + 2 + k) * kThreads];
      r[kRecShadow + 2 + k] = px[(kPxVis + 2 + k) * kThreads];
    }
  }
  if (phase != 0u) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      r[kRecCsv + k] = px[(kPxCsv + k) * kThreads];
      r[kRecNrm + k] = px[(kPxNrm + k) * kThreads];
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) r[kRecCol + k] = px[(kPxCol + k) * kThreads];
  }
}

// Texel and normal of the primary leaf (ns, nd) at `level`: the leaf fetch of
// Walker::leaf (octree_fsh.c:218-247), the dynamic model winning where it
// holds the leaf; dyn: the render walked a dynamic tree.
__device__ __forceinline__ void leaf_texel(const DevScene& sc, bool dyn, int32_t ns, int32_t nd, int level,
                                           float4& col, float4& nrm) {
  bool oob = false;  // (the walk that found the leaf reported it)
  const int32_t ms = load_model(sc.tree[0], ns, level, oob);
  const int32_t md = dyn ? load_model(sc.tree[1], nd, level, oob) : 0;
  load_attr(sc.model[0], ms, col, nrm, oob);
  if (md > 0) load_attr(sc.model[1], md, col, nrm, oob);
}

// kSplitStatic: the lanes whose new ray is not walked (defer) hand their
// pixel, its state words px (stride kThreads) and the phase to resume at, to
// the two-tree kernel: one atomic per warp. Out of line: it runs once per
// handed-on ray, away from the walk's hot code.
static __device__ __noinline__ void hand_on(bool defer, int phase, uint32_t* px, const Wave& wave) {
  const unsigned dm = __ballot_sync(0xFFFFFFFFu, defer);
  const int lead = __ffs((int)dm) - 1;
  unsigned base = 0;
  if ((int)(threadIdx.x & 31u) == lead) base = atomicAdd(wave.qcount, (unsigned)__popc(dm));
  base = __shfl_sync(0xFFFFFFFFu, base, lead);
  if (!defer) return;
  const unsigned q = base + __popc(dm & lanemask_lt());
  if (q >= wave.cap) {
    atomicOr(wave.err, kErrRecordOverflow);  // wave.stop leaves room for every pixel in flight
    return;
  }
  write_record(wave.rec + (size_t)q * kSplitRecWords, px, (uint32_t)phase);
}

template <bool EXACT, bool DYN, int MODE, bool PROP>
struct Shader {
  const DevScene& sc;
  const Batch& batch;
  const Wave& wave;
  Stack st;
  PixRef px;
  Walker<EXACT, DYN, PROP> w;
  int phase;     // kind of the lane's current ray, kIdle without a pixel
  bool running;  // the ray is being walked
  bool enqueue;  // primary pass: the pixel goes to the shade pass
  int result;    // status of the ray once it ended
  int maxlevel;
  int prop_k;    // next proposal to try
  uint32_t rec_q;  // shade pass: record of the pixel
  uint32_t next_target;
  int next_tdepth;
  float4 bc;
  unsigned long long stat[kStatCount];

  __device__ __forceinline__ const qbc_view& view() const { return batch.job[px.w(kPxView)].v; }

  // Index of the pixel among all pixels of the batch (views in order).
  __device__ __forceinline__ int64_t pixel_index() const {
    const ViewJob& J = batch.job[px.w(kPxView)];
    const uint32_t xy = px.w(kPxXY);
    return J.pixel_begin + (int64_t)(xy >> 16) * J.v.width_px + (xy & 0xFFFFu);
  }

  __device__ __forceinline__ void write_out(float4 col) {
    const ViewJob& J = batch.job[px.w(kPxView)];
    uint32_t xy = px.w(kPxXY);
    int i = (int)(xy & 0xFFFFu), j = (int)(xy >> 16);
    const int64_t o = (int64_t)j * J.v.width_px + i;
    const qbc_outputs& out = J.o;
    if (out.rgba8)
      reinterpret_cast<uint32_t*>(out.rgba8)[o] =
          unorm8(col.x) | (unorm8(col.y) << 8) | (unorm8(col.z) << 16) | (unorm8(col.w) << 24);
    if (out.rgba32f) reinterpret_cast<float4*>(out.rgba32f)[o] = col;
    if (out.flags) out.flags[o] = px.w(kPxFlags) & ~kWantFlare;
    if (out.leaf)
      reinterpret_cast<int4*>(out.leaf)[o] = make_int4((int32_t)px.w(kPxLeaf), (int32_t)px.w(kPxLeaf + 1),
                                                       (int32_t)px.w(kPxLeaf + 2), (int32_t)px.w(kPxLeaf + 3));
    if (out.isp)
      reinterpret_cast<float4*>(out.isp)[o] =
          make_float4(px.f(kPxIsp), px.f(kPxIsp + 1), px.f(kPxIsp + 2), px.f(kPxIsp + 3));
    if (out.visits)
      reinterpret_cast<uint4*>(out.visits)[o] =
          make_uint4(px.w(kPxVis), px.w(kPxVis + 1), px.w(kPxVis + 2), px.w(kPxVis + 3));
    phase = kIdle;
  }

  __device__ __forceinline__ void discard() {
    px.w(kPxFlags) |= QBC_PX_DISCARD;
    write_out(make_float4(0.0f, 0.0f, 0.0f, 0.0f));
  }

  // Pixel (i, j) of view vi: ray generation (octree_fsh.c:402-418). Sets the
  // primary ray into (rp, rd).
  __device__ __forceinline__ void begin_pixel(int vi, int i, int j, float3& rp, float3& rd) {
    px.w(kPxView) = (uint32_t)vi;
    px.w(kPxXY) = (uint32_t)i | ((uint32_t)j << 16);
    const qbc_view& v = batch.job[vi].v;
    maxlevel = v.maxlevel;
    bc = held_bc<EXACT>(v);
    const float4 ray = camera_ray(v, i, j);
    const float3 csv = make_float3(ray.x, ray.y, ray.z);
    px.w(kPxFlags) = flare_wanted(v, ray.w) ? kWantFlare : 0u;
    px.f(kPxCsv) = csv.x;
    px.f(kPxCsv + 1) = csv.y;
    px.f(kPxCsv + 2) = csv.z;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      px.w(kPxLeaf + k) = (uint32_t)-1;
      px.w(kPxVis + k) = 0u;
      px.f(kPxIsp + k) = 0.0f;
    }
    phase = kPrimary;
    rp = make_float3(v.camfp[0], v.camfp[1], v.camfp[2]);
    rd = csv;
  }

  // Shadow ray of the pixel in smem: from the light to the primary hit.
  __device__ __forceinline__ void shadow_ray(float3& rp, float3& rd) const {
    const qbc_view& v = view();
    rp = make_float3(v.light[0], v.light[1], v.light[2]);
    rd = make_float3(px.f(kPxIsp) - rp.x, px.f(kPxIsp + 1) - rp.y, px.f(kPxIsp + 2) - rp.z);
  }

  // The next usable proposal from prop_k on: the level-pdepth cell around
  // the proposed point of the shadow ray. Returns false when none is left.
  // (Launches without PROP have wave.nprop 0: the proposal words, which
  // their kernels do not keep, are never read.)
  __device__ __forceinline__ bool next_proposal(float3 rp, float3 rd) {
    while (prop_k < wave.nprop) {
      const float t = px.f(kPxProp + prop_k);
      ++prop_k;
      if (!(t > 0.0f && t < 1.0f)) continue;
      const float3 q = make_float3(rp.x + rd.x * t, rp.y + rd.y * t, rp.z + rd.z * t);
      const float s = bc.w;
      if (!(q.x >= bc.x && q.x < bc.x + s && q.y >= bc.y - s && q.y < bc.y && q.z >= bc.z - s && q.z < bc.z)) continue;
      if (bc.x != 0.0f || bc.y != s || bc.z != s) return false;  // paths assume basecube (0, S, S, S)
      next_tdepth = min(wave.pdepth, maxlevel);
      next_target = point_path(q, s, next_tdepth);
      return true;
    }
    return false;
  }

  // Shade pass: the pixel of record q; sets its first ray into (rp, rd). The
  // camera ray, the primary texel and normal are recomputed, as begin_pixel
  // and the primary leaf fetch made them. A split frame's two-tree kernel
  // resumes the pixel from its record's state at the ray it stopped at.
  __device__ __forceinline__ void begin_record(uint32_t q, float3& rp, float3& rd) {
    constexpr int kStride = MODE == kSplitFinish ? kSplitRecWords : kRecWords;
    const uint32_t* r = wave.rec + (size_t)q * kStride;
    rec_q = q;
    const uint32_t vw = r[kRecView], xy = r[kRecXY];
    const int ph = MODE == kSplitFinish ? (int)(vw >> 8) : 0;
    if (MODE != kSplitFinish || ph == kPrimary) {
      begin_pixel((int)(vw & 0xFFu), (int)(xy & 0xFFFFu), (int)(xy >> 16), rp, rd);
      if (MODE == kSplitFinish) return;
    } else {
      px.w(kPxView) = vw & 0xFFu;
      px.w(kPxXY) = xy;
      const qbc_view& v = view();
      maxlevel = v.maxlevel;
      bc = held_bc<EXACT>(v);
    }
    const uint32_t flags = r[kRecFlags];
    px.w(kPxFlags) = flags;
#pragma unroll
    for (int k = 0; k < 4; ++k) px.w(kPxIsp + k) = r[kRecIsp + k];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      px.w(kPxLeaf + k) = r[kRecLeaf + k];
      px.w(kPxVis + k) = r[kRecVis + k];
      px.w(kPxLeaf + 2 + k) = MODE == kSplitFinish && ph == kFlare ? r[kRecShadow + k] : (uint32_t)-1;
      px.w(kPxVis + 2 + k) = MODE == kSplitFinish && ph == kFlare ? r[kRecShadow + 2 + k] : 0u;
    }
    prop_k = 0;
    next_tdepth = 0;
    if (MODE == kSplitFinish) {
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        px.w(kPxCsv + k) = r[kRecCsv + k];
        px.w(kPxNrm + k) = r[kRecNrm + k];
      }
#pragma unroll
      for (int k = 0; k < 4; ++k) px.w(kPxCol + k) = r[kRecCol + k];
      if (ph == kShadow) {
        shadow_ray(rp, rd);
        phase = kShadow;
      } else {
        start_flare(rp, rd);
      }
      return;
    }
    float4 col = make_float4(0.0f, 0.0f, 0.0f, 0.0f), nrm = col;
    if (flags & QBC_PX_PRIMARY_LEAF)
      leaf_texel(sc, DYN, (int32_t)r[kRecLeaf], (int32_t)r[kRecLeaf + 1], maxlevel, col, nrm);
#pragma unroll
    for (int k = 0; k < 4; ++k) px.f(kPxCol + k) = (&col.x)[k];
    if (flags & QBC_PX_SHADED) {
      px.f(kPxNrm) = nrm.x;
      px.f(kPxNrm + 1) = nrm.y;
      px.f(kPxNrm + 2) = nrm.z;
    }
#pragma unroll
    for (int k = 0; k < 3; ++k)
      if (PROP) px.w(kPxProp + k) = r[kRecProp + k];
    if (flags & QBC_PX_SHADED) {
      shadow_ray(rp, rd);
      phase = kShadow;
      if (PROP && next_proposal(rp, rd)) phase = kProposal;
    } else {
      start_flare(rp, rd);
    }
  }

  __device__ __forceinline__ void start_flare(float3& rp, float3& rd) {
    px.w(kPxFlags) |= QBC_PX_FLARE_TEST;
    const qbc_view& v = view();
    rp = make_float3(v.camfp[0], v.camfp[1], v.camfp[2]);
    rd = make_float3(v.light[0] - rp.x, v.light[1] - rp.y, v.light[2] - rp.z);
    phase = kFlare;
  }

  // Flare ray (octree_fsh.c:452-459) if the pixel wants one: returns true and
  // sets (rp, rd); otherwise writes the pixel.
  __device__ __forceinline__ bool flare_or_finish(float4 col, float3& rp, float3& rd) {
    if (px.w(kPxFlags) & kWantFlare) {
#pragma unroll
      for (int k = 0; k < 4; ++k) px.f(kPxCol + k) = (&col.x)[k];
      start_flare(rp, rd);
      return true;
    }
    write_out(col);
    return false;
  }

  // Shading of octree_fsh.c:436-449 with the shadow walk's lit value.
  __device__ __forceinline__ float4 shade(float lit) {
    const qbc_view& v = view();
    float4 pi = make_float4(px.f(kPxIsp), px.f(kPxIsp + 1), px.f(kPxIsp + 2), px.f(kPxIsp + 3));
    float4 pc = make_float4(px.f(kPxCol), px.f(kPxCol + 1), px.f(kPxCol + 2), px.f(kPxCol + 3));
    float3 pn = make_float3(px.f(kPxNrm), px.f(kPxNrm + 1), px.f(kPxNrm + 2));
    float3 csv = make_float3(px.f(kPxCsv), px.f(kPxCsv + 1), px.f(kPxCsv + 2));
    float3 lghtv = make_float3(pi.x - v.light[0], pi.y - v.light[1], pi.z - v.light[2]);
    float3 nl = normalize3(make_float3(-lghtv.x, -lghtv.y, -lghtv.z));
    float3 nn = normalize3(pn);
    float3 nc = normalize3(make_float3(-csv.x, -csv.y, -csv.z));
    float lght_nrm_ang = glsl_max(dot3(nl, nn), 0.0f);
    float camv_nrm_ang = glsl_max(dot3(nc, nn), 0.0f);
    if (lit != 0.0f) px.w(kPxFlags) |= QBC_PX_LIT;
    float k = 0.1f + 0.2f * camv_nrm_ang + lght_nrm_ang * lit * 0.7f;
    pc.x = pc.x * k;
    pc.y = pc.y * k;
    pc.z = pc.z * k;
    pc.z *= 0.7f;
    float g = (float)v.shoot * camv_nrm_ang * 0.1f;
    pc.x += g;
    pc.y += g;
    pc.z += g;
    return pc;
  }

  // The lane's ray ended with `result`: record it and decide the pixel's next
  // ray. Returns true with (rp, rd) set when another ray of this pixel starts.
  __device__ __forceinline__ bool consume(float3& rp, float3& rd) {
    const int r = result;
    float4 col = make_float4(0.f, 0.f, 0.f, 0.f), nrm = col, isp = col;
    if (r == kLeaf) {
      int32_t ms, md;
      w.leaf(sc, ms, md, col, nrm);
      isp = w.e;
    }

    if (phase == kProposal) {
      // a proposal walk ended: a leaf well before the hit proves the shadow
      stat[kStatPropTried] += 1;
      stat[kStatPropVisits] += w.vis_s + w.vis_d;
      px.w(kPxVis + 2) += w.vis_s;
      px.w(kPxVis + 3) += w.vis_d;
      bool proven = false;
      if (r == kLeaf) {
        float dx = isp.x - px.f(kPxIsp), dy = isp.y - px.f(kPxIsp + 1), dz = isp.z - px.f(kPxIsp + 2);
        proven = isp.w < 1.0f && dx * dx + dy * dy + dz * dz > 16.0f;
      }
      if (proven) {
        stat[kStatPropProven] += 1;
        // the plain walk reaches a leaf at least this far from the hit: unlit
        px.w(kPxFlags) |= QBC_PX_SHADOW_LEAF;
        px.w(kPxLeaf + 2) = (uint32_t)-2;  // the plain walk's leaf was not computed
        px.w(kPxLeaf + 3) = (uint32_t)-2;
        return flare_or_finish(shade(0.0f), rp, rd);
      }
      shadow_ray(rp, rd);
      if (next_proposal(rp, rd)) return true;  // phase stays kProposal
      phase = kShadow;
      return true;
    }

    if (w.oob) px.w(kPxFlags) |= QBC_PX_OOB;

    if (phase == kPrimary) {
      px.w(kPxVis) = w.vis_s;
      px.w(kPxVis + 1) = w.vis_d;
      if (r == kLeaf) {
        px.w(kPxFlags) |= QBC_PX_PRIMARY_LEAF;
        px.w(kPxLeaf) = (uint32_t)w.ns;
        px.w(kPxLeaf + 1) = (uint32_t)w.nd;
      }
      px.f(kPxIsp) = isp.x;
      px.f(kPxIsp + 1) = isp.y;
      px.f(kPxIsp + 2) = isp.z;
      px.f(kPxIsp + 3) = isp.w;
#pragma unroll
      for (int k = 0; k < 4; ++k) px.f(kPxCol + k) = (&col.x)[k];
      if (isp.w > 0.0f) {
        px.w(kPxFlags) |= QBC_PX_SHADED;
        px.f(kPxNrm) = nrm.x;
        px.f(kPxNrm + 1) = nrm.y;
        px.f(kPxNrm + 2) = nrm.z;
        if (MODE == kPrimaryPass) {
          enqueue = true;
          return false;
        }
        // shadow ray from the light to the hit (octree_fsh.c:431-432)
        shadow_ray(rp, rd);
        phase = kShadow;
        return true;
      }
      if (MODE == kPrimaryPass && (px.w(kPxFlags) & kWantFlare)) {
        enqueue = true;
        return false;
      }
      return flare_or_finish(col, rp, rd);
    }
    if (phase == kShadow) {
      // shading (octree_fsh.c:433-449)
      stat[kStatShadowRays] += 1;
      stat[kStatShadowVisits] += w.vis_s + w.vis_d;
      px.w(kPxVis + 2) += w.vis_s;
      px.w(kPxVis + 3) += w.vis_d;
      if (r == kLeaf) {
        px.w(kPxFlags) |= QBC_PX_SHADOW_LEAF;
        px.w(kPxLeaf + 2) = (uint32_t)w.ns;
        px.w(kPxLeaf + 3) = (uint32_t)w.nd;
      }
      float ix = isp.x - px.f(kPxIsp), iy = isp.y - px.f(kPxIsp + 1), iz = isp.z - px.f(kPxIsp + 2);
      float sqr = ix * ix + iy * iy + iz * iz;
      float lit = (15.0f < sqr) ? 0.0f : 1.0f;  // step(sqr, 15.0)
      if (MODE == kShadePass && wave.log) {
        uint32_t* rq = wave.rec + (size_t)rec_q * kRecWords;
        const float lt = r == kLeaf ? isp.w : -1.0f;
        reinterpret_cast<float&>(rq[kRecLogT]) = lt;
        rq[kRecLogLit] = lit != 0.0f ? 1u : 0u;
        if (wave.pixlog) wave.pixlog[pixel_index()] = lit != 0.0f ? -1.0f : lt;
      }
      return flare_or_finish(shade(lit), rp, rd);
    }
    // flare ray ended (octree_fsh.c:456-458)
    const qbc_view& v = view();
    float4 pc = make_float4(px.f(kPxCol), px.f(kPxCol + 1), px.f(kPxCol + 2), px.f(kPxCol + 3));
    float resv_x = isp.x - v.camfp[0];
    float lx = v.light[0] - v.camfp[0];
    if (resv_x / lx > 1.0f) {
      px.w(kPxFlags) |= QBC_PX_FLARE_WHITE;
      pc = make_float4(1.0f, 1.0f, 1.0f, 1.0f);
    }
    write_out(pc);
    return false;
  }
};

// Global tile queue: 32-pixel warp tiles (8x4 by default), numbered view by
// view.
__device__ __forceinline__ int tile_view(const Batch& b, int tile) {
  int lo = 0, hi = b.n - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (b.job[mid].tile_begin <= tile)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// Lanes whose ray ended wait until at least batch.service_min lanes of the
// warp need service (or no ray is left running); then ray transitions,
// refills and ray starts run for all of them together instead of one lane at
// a time.
constexpr int kServiceMinDefault = 4;

// MODE kFused: every pixel's primary ray, shadow ray, shading and flare.
// MODE kPrimaryPass: primary rays only; shaded and flare pixels go to the
// record queue (warp-aggregated atomics), the rest are written.
// MODE kShadePass: the queued pixels' shadow rays (first the proposals, with
// PROP), shading and flare.
// A fused frame with two trees may run split, as two launches:
// MODE kSplitStatic (the one-tree kernel): as kFused, but a ray whose
// two-tree walk would read the dynamic tree (Walker::walks_dynamic) is not
// walked: its pixel goes with its state to the record queue. The other
// rays' two-tree walks read the static tree alone, so the one-tree walk
// gives them the same results with the lighter kernel. Once the queue may
// not hold every pixel the warps can still hand on (wave.stop), no warp
// takes a new tile.
// MODE kSplitFinish (the two-tree kernel): the queued pixels, each from the
// ray it stopped at, then the tiles the one-tree kernel left.
// Minimum resident blocks per SM the register allocation must allow: the
// walk is latency-bound per warp, so more resident warps pay as long as
// nothing (or next to nothing) spills: 6 (80 registers) for the fused,
// primary-pass and split kernels; the shade passes, which also shade and
// test proposals, and the two-tree walk of an inexact basecube (which keeps
// the node blocks live) keep 5 with both trees and no bound with one.
template <bool EXACT, bool DYN, int MODE>
constexpr int render_min_blocks() {
  return (MODE == kShadePass || (DYN && !EXACT)) ? (DYN ? 5 : 1) : 6;
}

template <bool EXACT, bool DYN, int MODE, bool PROP>
__global__ void __launch_bounds__(kThreads, render_min_blocks<EXACT, DYN, MODE>()) render_kernel(DevScene sc, const __grid_constant__ Batch batch,
                                                          unsigned int* queue, const __grid_constant__ Wave wave) {
  extern __shared__ uint32_t smem[];
  const int tid = threadIdx.x, lane = tid & 31;
  constexpr int kW = Walker<EXACT, DYN, PROP>::kWords;
  constexpr bool kRecords = MODE == kShadePass || MODE == kSplitFinish;
  Shader<EXACT, DYN, MODE, PROP> S{sc, batch, wave, Stack{smem + tid, kThreads},
                                   PixRef{smem + kW * batch.max_level * kThreads + tid}};
  S.phase = kIdle;
  S.running = false;
  S.enqueue = false;
  S.result = 0;
  S.maxlevel = 0;
  S.prop_k = 0;
  S.rec_q = 0;
  S.next_target = 0;
  S.next_tdepth = 0;
  S.bc = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
  for (int k = 0; k < kStatCount; ++k) S.stat[k] = 0;
  int chunk = 0, consumed = 32;  // warp-uniform
  bool fast = false;             // warp-uniform: see the service phase
  bool exhausted = false;
  bool from_rec = kRecords;      // warp-uniform: the chunk is 32 records (else a tile)
  const unsigned nrec = kRecords ? min(*wave.qcount, wave.cap) : 0u;
  const unsigned ntiles = (unsigned)batch.tiles_total;

  for (;;) {
    const unsigned run = __ballot_sync(0xFFFFFFFFu, S.running);
    const int waiting = 32 - __popc(run);
    if (run == 0 || waiting >= batch.service_min) {
      // ---- service: consume ended rays, refill, start new rays together ----
      float3 rp = make_float3(0.f, 0.f, 0.f), rd = rp;
      bool go = false;
      if (!S.running && S.phase != kIdle) go = S.consume(rp, rd);
      if (MODE == kPrimaryPass) {
        // hand shaded / flare pixels to the shade pass: one atomic per warp
        const unsigned enq = __ballot_sync(0xFFFFFFFFu, S.enqueue);
        if (enq) {
          unsigned base = 0;
          if (lane == __ffs(enq) - 1) base = atomicAdd(wave.qcount, (unsigned)__popc(enq));
          base = __shfl_sync(0xFFFFFFFFu, base, __ffs(enq) - 1);
          if (S.enqueue) {
            const unsigned q = base + __popc(enq & lanemask_lt());
            if (q < wave.cap) write_record(wave.rec + (size_t)q * kRecWords, S.px.base, 0u);
            S.enqueue = false;
            S.phase = kIdle;
          }
        }
      }
      unsigned idle = __ballot_sync(0xFFFFFFFFu, S.phase == kIdle);
      while (idle && !exhausted) {
        if (consumed >= 32) {
          unsigned t0 = 0, stop = 0;
          if (lane == 0) {
            if (MODE == kSplitStatic) stop = *(volatile unsigned*)wave.qcount > wave.stop ? 1u : 0u;
            if (!stop) t0 = atomicAdd(from_rec ? wave.qnext : queue, from_rec ? 32u : 1u);
          }
          if (MODE == kSplitStatic && __shfl_sync(0xFFFFFFFFu, stop, 0)) {
            exhausted = true;
            break;
          }
          chunk = (int)__shfl_sync(0xFFFFFFFFu, t0, 0);
          consumed = 0;
          if (MODE == kSplitFinish && from_rec && (unsigned)chunk >= nrec) {
            from_rec = false;  // records done: the tiles left
            consumed = 32;
            continue;
          }
          if ((unsigned)chunk >= (from_rec ? nrec : ntiles)) {
            exhausted = true;
            break;
          }
        }
        const int avail = 32 - consumed;
        const int rank = __popc(idle & lanemask_lt());
        if (((idle >> lane) & 1u) && rank < avail) {
          const int slot = consumed + rank;
          if (from_rec) {
            const unsigned q = (unsigned)chunk + slot;
            if (q < nrec) {
              S.begin_record(q, rp, rd);
              go = true;
            }
          } else {
            const int vi = tile_view(batch, chunk);
            const ViewJob& J = batch.job[vi];
            const int t = chunk - J.tile_begin;
            const int sh = batch.tile_shift;
            const int x = ((t % J.tiles_x) << sh) + (slot & ((1 << sh) - 1));
            const int y = (t / J.tiles_x) * (32 >> sh) + (slot >> sh);
            if (x < J.v.width_px && y < J.v.height_px) {
              S.begin_pixel(vi, x, y, rp, rd);
              go = true;
            }
          }
        }
        consumed += min(avail, __popc(idle));
        idle = __ballot_sync(0xFFFFFFFFu, S.phase == kIdle);
      }
      bool defer = false;  // kSplitStatic: the new ray's two-tree walk would read the dynamic tree
      if (go) {
        if (S.w.start(S.bc, rp, rd, sc, S.maxlevel) == kDiscard) {
          S.discard();
        } else if (MODE == kSplitStatic && S.w.walks_dynamic(sc, S.bc, S.maxlevel)) {
          defer = true;
        } else {
          S.running = true;
          if (PROP && S.phase == kProposal) {
            S.w.target = S.next_target;
            S.w.tdepth = S.next_tdepth;
          }
        }
      }
      if (MODE == kSplitStatic && __any_sync(0xFFFFFFFFu, defer)) {
        hand_on(defer, S.phase, S.px.base, wave);
        if (defer) S.phase = kIdle;
      }
      // whether every running lane may divide by its reciprocals (the set
      // of running rays changes only here)
      fast = EXACT && __all_sync(0xFFFFFFFFu, !S.running || (S.w.mode & 1u));
      if (exhausted && __ballot_sync(0xFFFFFFFFu, S.phase != kIdle) == 0) break;
    }
    if (S.running) {
      const int r = S.w.step(sc, S.maxlevel, S.bc, S.st, fast);
      if (r != kRunning) {
        S.running = false;
        S.result = r;
      }
    }
  }
  if (MODE == kSplitFinish && blockIdx.x == 0 && tid == 0) atomicAdd(wave.stats + kStatSplitQueued, nrec);
  if (MODE == kShadePass) {
    // statistics: one atomic per warp and counter
#pragma unroll
    for (int k = 0; k < kStatCount; ++k) {
      unsigned long long v = S.stat[k];
      for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xFFFFFFFFu, v, o);
      if (lane == 0 && v) atomicAdd(wave.stats + k, v);
    }
  }
}

// The plain schedule (QBC_OPT_PERSISTENT 0): one thread per pixel for its
// whole life (primary ray, shadow ray, shading, flare), one warp per 32-pixel
// tile, no work queue and no batched service; a lane whose pixel is done
// idles until its warp's last pixel is. Same walker and shader code as
// render_kernel, so the same pixels; kept as the baseline the persistent
// kernel is measured against.
template <bool EXACT, bool DYN>
__global__ void __launch_bounds__(kThreads, render_min_blocks<EXACT, DYN, kFused>()) simple_kernel(DevScene sc, const __grid_constant__ Batch batch) {
  extern __shared__ uint32_t smem[];
  const int tid = threadIdx.x;
  const int tile = (int)((blockIdx.x * (unsigned)kThreads + tid) >> 5);
  if (tile >= batch.tiles_total) return;
  constexpr int kW = Walker<EXACT, DYN, false>::kWords;
  const Wave wave{};
  Shader<EXACT, DYN, kFused, false> S{sc, batch, wave, Stack{smem + tid, kThreads},
                                      PixRef{smem + kW * batch.max_level * kThreads + tid}};
  S.running = false;
  S.enqueue = false;
  S.prop_k = 0;
  S.rec_q = 0;
  S.next_target = 0;
  S.next_tdepth = 0;
  const int vi = tile_view(batch, tile);
  const ViewJob& J = batch.job[vi];
  const int t = tile - J.tile_begin, slot = tid & 31, sh = batch.tile_shift;
  const int x = ((t % J.tiles_x) << sh) + (slot & ((1 << sh) - 1));
  const int y = (t / J.tiles_x) * (32 >> sh) + (slot >> sh);
  if (x >= J.v.width_px || y >= J.v.height_px) return;
  float3 rp, rd;
  S.begin_pixel(vi, x, y, rp, rd);
  for (;;) {
    if (S.w.start(S.bc, rp, rd, sc, S.maxlevel) == kDiscard) {
      S.discard();
      return;
    }
    const bool fast = EXACT && (S.w.mode & 1u);
    int r;
    do {
      r = S.w.step(sc, S.maxlevel, S.bc, S.st, fast);
    } while (r == kRunning);
    S.result = r;
    if (!S.consume(rp, rd)) return;
  }
}

struct RayJob {
  const float* pos;
  const float* dir;
  int64_t n;
  float4 bc;
  int32_t maxlevel;
  int32_t service_min;  // waiting lanes that start a service (1..32)
  qbc_ray_hits o;
};

// Batched ray queries (qbc_trace_rays), on the render kernel's schedule: a
// lane walks a sequence of rays (grid stride); a lane whose ray ended waits
// until service_min lanes of its warp wait (or none runs), then they write
// their results and start their next rays together, and the warp votes on
// the division by reciprocals for the rays now running.
template <bool EXACT, bool DYN>
__global__ void __launch_bounds__(kThreads) rays_kernel(DevScene sc, const __grid_constant__ RayJob job) {
  extern __shared__ uint32_t smem[];
  Stack st{smem + threadIdx.x, kThreads};
  Walker<EXACT, DYN> w;
  const int64_t stride = (int64_t)gridDim.x * kThreads;
  int64_t i = blockIdx.x * (int64_t)kThreads + threadIdx.x;  // the lane's current ray
  int r = kMiss;
  bool running = false, ended = false;  // ended: ray i is done and not yet written
  bool fast = false;                    // warp-uniform
  for (;;) {
    const unsigned run = __ballot_sync(0xFFFFFFFFu, running);
    if (run == 0u || 32 - __popc(run) >= job.service_min) {
      if (!running) {
        for (;;) {
          if (ended) {
            int32_t ms = -1, md = -1, ls = -1, ld = -1;
            float4 col = make_float4(0.f, 0.f, 0.f, 0.f), nrm = col, isp = col;
            if (r == kLeaf) {
              w.leaf(sc, ms, md, col, nrm);
              isp = w.e;
              ls = w.ns;
              ld = w.nd;
            }
            const qbc_ray_hits& o = job.o;
            if (o.status) o.status[i] = r == kDiscard ? kDiscard : (r == kLeaf ? kLeaf : kMiss);
            if (o.leaf) reinterpret_cast<int2*>(o.leaf)[i] = make_int2(ls, ld);
            if (o.model) reinterpret_cast<int2*>(o.model)[i] = make_int2(ms, md);
            if (o.isp) reinterpret_cast<float4*>(o.isp)[i] = isp;
            if (o.col) reinterpret_cast<float4*>(o.col)[i] = col;
            if (o.nrm) reinterpret_cast<float4*>(o.nrm)[i] = nrm;
            if (o.visits)
              reinterpret_cast<uint2*>(o.visits)[i] = r == kDiscard ? make_uint2(0, 0) : make_uint2(w.vis_s, w.vis_d);
            ended = false;
            i += stride;
          }
          if (i >= job.n) break;
          const float3 p = make_float3(job.pos[3 * i], job.pos[3 * i + 1], job.pos[3 * i + 2]);
          const float3 d = make_float3(job.dir[3 * i], job.dir[3 * i + 1], job.dir[3 * i + 2]);
          r = w.start(job.bc, p, d, sc, job.maxlevel);
          if (r != kDiscard) {
            running = true;
            break;
          }
          ended = true;  // written on the next pass of this loop
        }
      }
      if (__ballot_sync(0xFFFFFFFFu, running) == 0u) break;  // no ray left for any lane
      fast = EXACT && __all_sync(0xFFFFFFFFu, !running || (w.mode & 1u));
    }
    if (running) {
      r = w.step(sc, job.maxlevel, job.bc, st, fast);
      if (r != kRunning) {
        running = false;
        ended = true;
      }
    }
  }
}

}  // namespace qbc
