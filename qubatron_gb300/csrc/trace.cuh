// Device traversal of qubatron's sparse octree: the joint static + dynamic
// `cube_trace_line` of src/qubatron/shaders/octree_fsh.c:138-379, restated for
// one thread per ray with a compact stack.
//
// Results are bit-identical to the shader's FP32 arithmetic: this file must be
// compiled with -fmad=false (no fused multiply-add), IEEE division and sqrt and
// no flush-to-zero, and every expression keeps the shader's operation order.
//
// Stack. The shader keeps per level a cube, four candidate points, four octets
// and three ints (~1.9 KB per thread, octree_fsh.c:50-58). Here a level keeps
// three 32-bit words in shared memory:
//   word 0: the sorted candidate list, 4 x 5 bits (octet | source << 3), its
//           length (bits 20-22) and the index of the next candidate (23-25);
//           source 0 is the cube's entry point, 1/2/3 the hit of the z/x/y
//           bisecting plane of that cube;
//   word 1, 2: the level's node index in the static and dynamic tree.
// A candidate point is recomputed from its source with the same operations on
// the same inputs, so it has the same bits as the stored one. The cube of a
// level is recovered on the way up by undoing the child shift, which is exact
// when every cube coordinate is representable (checked on the host, EXACT =
// true), or else by replaying the path from the root.
#pragma once

#include <cstdint>

namespace qbc {

constexpr float kFltMax = 3.402823466e+38f;  // FLT_MAX (octree_fsh.c:60)
// Bound on node entries per ray: a valid tree needs far fewer, a corrupt one
// with repeating child indices could make the walk exponential. Past it the
// ray ends as a miss flagged out-of-range, exactly as the oracle does.
constexpr int kMaxPushes = 1 << 22;

struct DevTree {
  const int4* child;     // 2 int4 per node: the 8 child indices
  const int32_t* model;  // slot 8: model index of the point that made the node
  int64_t n;             // nodes held; index >= n reads as 0 and is reported
};

struct DevModel {
  const float4* col;  // (r, g, b, 1) per point, as an RGB32F texel reads
  const float4* nrm;  // (x, y, z, 1)
  int64_t n;
};

struct DevScene {
  DevTree tree[2];    // 0 static, 1 dynamic
  DevModel model[2];
};

enum : int { kMiss = 0, kLeaf = 1, kDiscard = 2 };

struct TraceOut {
  float4 isp;      // entry point of the leaf cell, w = t
  float4 col;
  float4 nrm;
  int32_t leaf_s, leaf_d;
  int32_t model_s, model_d;
  int status;
  uint32_t vis_s, vis_d;  // subnode tests with a non-empty node, per tree
  bool oob;
};

// ---- is_cube_{x,y,z}plane (octree_fsh.c:62-99) ----
__device__ __forceinline__ float4 hit_xplane(float x, float3 p, float3 d) {
  float4 r = make_float4(kFltMax, kFltMax, kFltMax, kFltMax);
  if (d.x != 0.0f) {
    r.w = (x - p.x) / d.x;
    r.y = p.y + d.y * r.w;
    r.z = p.z + d.z * r.w;
    r.x = x;
  }
  return r;
}
__device__ __forceinline__ float4 hit_yplane(float y, float3 p, float3 d) {
  float4 r = make_float4(kFltMax, kFltMax, kFltMax, kFltMax);
  if (d.y != 0.0f) {
    r.w = (y - p.y) / d.y;
    r.x = p.x + d.x * r.w;
    r.z = p.z + d.z * r.w;
    r.y = y;
  }
  return r;
}
__device__ __forceinline__ float4 hit_zplane(float z, float3 p, float3 d) {
  float4 r = make_float4(kFltMax, kFltMax, kFltMax, kFltMax);
  if (d.z != 0.0f) {
    r.w = (z - p.z) / d.z;
    r.x = p.x + d.x * r.w;
    r.y = p.y + d.y * r.w;
    r.z = z;
  }
  return r;
}

// Half-open face tests (octree_fsh.c:166-192, 263-271).
__device__ __forceinline__ bool in_zface(float4 a, float4 t, float4 b) {
  return t.x < a.x && a.x <= b.x && t.y > a.y && a.y >= b.y;
}
__device__ __forceinline__ bool in_xface(float4 a, float4 t, float4 b) {
  return t.y > a.y && a.y >= b.y && t.z > a.z && a.z >= b.z;
}
__device__ __forceinline__ bool in_yface(float4 a, float4 t, float4 b) {
  return t.x < a.x && a.x <= b.x && t.z > a.z && a.z >= b.z;
}

__device__ __forceinline__ float4 brb_of(float4 t) {
  return make_float4(t.x + t.w, t.y - t.w, t.z - t.w, 0.0f);
}
// hlf = brb + (tlf - brb) * 0.5 (octree_fsh.c:256)
__device__ __forceinline__ float3 hlf_of(float4 t) {
  float4 b = brb_of(t);
  return make_float3(b.x + (t.x - b.x) * 0.5f, b.y + (t.y - b.y) * 0.5f, b.z + (t.z - b.z) * 0.5f);
}

// Child cube of octet o (octree_fsh.c:342-347): x shifts right for bit 0,
// y down for bit 1, z back for bit 2.
__device__ __forceinline__ float4 child_cube(float4 t, int o) {
  float halfs = t.w / 2.0f;
  float kx = (o & 1) ? 1.0f : 0.0f, ky = (o & 2) ? 1.0f : 0.0f, kz = (o & 4) ? 1.0f : 0.0f;
  t.x += kx * halfs;
  t.y -= ky * halfs;
  t.z -= kz * halfs;
  t.w = halfs;
  return t;
}
// Inverse of child_cube; exact whenever the forward shift was.
__device__ __forceinline__ float4 parent_cube(float4 t, int o) {
  float hs = t.w;
  float kx = (o & 1) ? 1.0f : 0.0f, ky = (o & 2) ? 1.0f : 0.0f, kz = (o & 4) ? 1.0f : 0.0f;
  t.x -= kx * hs;
  t.y += ky * hs;
  t.z += kz * hs;
  t.w = hs * 2.0f;
  return t;
}

// Point of candidate source src (1 z, 2 x, 3 y bisecting plane) of cube t.
__device__ __forceinline__ float4 plane_point(int src, float4 t, float3 p, float3 d) {
  float3 h = hlf_of(t);
  if (src == 1) return hit_zplane(h.z, p, d);
  if (src == 2) return hit_xplane(h.x, p, d);
  return hit_yplane(h.y, p, d);
}

__device__ __forceinline__ int32_t pick8(int4 a, int4 b, int o) {
  int32_t lo = (o & 2) ? ((o & 1) ? a.w : a.z) : ((o & 1) ? a.y : a.x);
  int32_t hi = (o & 2) ? ((o & 1) ? b.w : b.z) : ((o & 1) ? b.y : b.x);
  return (o & 4) ? hi : lo;
}

// Child block of node i (oct_from_octets_for_index, octree_fsh.c:127-136):
// node 0 below the root is "no node"; a tree never uploaded holds nothing.
__device__ __forceinline__ bool load_block(const DevTree& t, int32_t i, int level, int4& a, int4& b,
                                           bool& oob) {
  a = make_int4(0, 0, 0, 0);
  b = a;
  if ((i == 0 && level > 0) || t.n == 0) return false;
  if (i < 0 || (int64_t)i >= t.n) {
    oob = true;
    return false;
  }
  a = __ldg(t.child + 2 * (int64_t)i);
  b = __ldg(t.child + 2 * (int64_t)i + 1);
  return true;
}

__device__ __forceinline__ int32_t load_child(const DevTree& t, int32_t i, int level, int o, bool& oob) {
  if ((i == 0 && level > 0) || t.n == 0) return 0;
  if (i < 0 || (int64_t)i >= t.n) {
    oob = true;
    return 0;
  }
  return __ldg(reinterpret_cast<const int32_t*>(t.child) + 8 * (int64_t)i + o);
}

__device__ __forceinline__ int32_t load_model(const DevTree& t, int32_t i, int level, bool& oob) {
  if ((i == 0 && level > 0) || t.n == 0) return 0;
  if (i < 0 || (int64_t)i >= t.n) {
    oob = true;
    return 0;
  }
  return __ldg(t.model + i);
}

__device__ __forceinline__ void load_attr(const DevModel& m, int32_t i, float4& col, float4& nrm, bool& oob) {
  col = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  nrm = col;
  if (m.n == 0) return;
  if (i < 0 || (int64_t)i >= m.n) {
    oob = true;
    return;
  }
  col = __ldg(m.col + i);
  nrm = __ldg(m.nrm + i);
}

// Per-thread stack in shared memory: word k of level l at st[(3 * l + k) * stride].
struct Stack {
  uint32_t* base;
  int stride;
  __device__ __forceinline__ uint32_t& at(int l, int k) const { return base[(3 * l + k) * stride]; }
};

__device__ __forceinline__ int list_len(uint32_t pk) { return (pk >> 20) & 7; }
__device__ __forceinline__ int list_next(uint32_t pk) { return (pk >> 23) & 7; }
__device__ __forceinline__ int list_entry(uint32_t pk, int k) { return (pk >> (5 * k)) & 31; }

// Cube and entry point of stack level `lv` by replaying the current path
// from the root: the same operations as the way down, so the same bits.
__device__ __forceinline__ void replay(const Stack& st, int lv, float4 bc, float4 e0, float3 p, float3 d,
                                       float4& cube, float4& e) {
  cube = bc;
  e = e0;
  for (int k = 0; k < lv; ++k) {
    uint32_t pk = st.at(k, 0);
    int c = list_entry(pk, list_next(pk) - 1);
    if (c >> 3) e = plane_point(c >> 3, cube, p, d);
    cube = child_cube(cube, c & 7);
  }
}

template <bool EXACT>
__device__ __noinline__ void trace(const DevScene& sc, float4 bc, int maxlevel, float3 p, float3 d,
                                   const Stack& st, TraceOut& r) {
  r.isp = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  r.col = r.isp;
  r.nrm = r.isp;
  r.leaf_s = -1;
  r.leaf_d = -1;
  r.model_s = -1;
  r.model_d = -1;
  r.status = kMiss;
  r.vis_s = 0;
  r.vis_d = 0;
  bool oob = false;

  // ---- basecube entry (octree_fsh.c:157-211) ----
  float4 cube = bc;
  float4 e0;  // entry point of the basecube
  {
    float4 cb = brb_of(cube);
    int hitc = 0;
    float4 h0 = make_float4(0.f, 0.f, 0.f, 0.f), h1 = h0, a;
#define QB_FACE(expr, test)       \
  a = expr;                       \
  if (test) {                     \
    if (hitc == 0) h0 = a;        \
    else if (hitc == 1) h1 = a;   \
    ++hitc;                       \
  }
    QB_FACE(hit_zplane(cube.z, p, d), in_zface(a, cube, cb))  // front
    QB_FACE(hit_zplane(cb.z, p, d), in_zface(a, cube, cb))    // back
    QB_FACE(hit_xplane(cube.x, p, d), in_xface(a, cube, cb))  // left
    QB_FACE(hit_xplane(cb.x, p, d), in_xface(a, cube, cb))    // right
    QB_FACE(hit_yplane(cube.y, p, d), in_yface(a, cube, cb))  // top
    QB_FACE(hit_yplane(cb.y, p, d), in_yface(a, cube, cb))    // bottom
#undef QB_FACE
    if (hitc < 2 || (h0.w < 0.0f && h1.w < 0.0f)) {
      r.status = kDiscard;
      return;
    }
    if (h1.w < h0.w) h0 = h1;
    if (h0.w < 0.0f) h0 = make_float4(p.x, p.y, p.z, 0.0f);
    e0 = h0;
  }

  float4 e = e0;  // entry point of the current cube
  int level = 0;
  int pushes = 0;
  int32_t ns = 0, nd = 0;

  for (;;) {
    if (level == maxlevel) {
      // ---- leaf (octree_fsh.c:218-247) ----
      int32_t ms = load_model(sc.tree[0], ns, level, oob);
      int32_t md = load_model(sc.tree[1], nd, level, oob);
      load_attr(sc.model[0], ms, r.col, r.nrm, oob);
      if (md > 0) load_attr(sc.model[1], md, r.col, r.nrm, oob);
      r.isp = e;
      r.leaf_s = ns;
      r.leaf_d = nd;
      r.model_s = ms;
      r.model_d = md;
      r.status = kLeaf;
      r.oob = oob;
      return;
    }

    // ---- subnode test of a freshly entered cube (octree_fsh.c:251-329) ----
    int4 s0, s1, d0, d1;
    if (load_block(sc.tree[0], ns, level, s0, s1, oob)) ++r.vis_s;
    if (load_block(sc.tree[1], nd, level, d0, d1, oob)) ++r.vis_d;

    float4 cb = brb_of(cube);
    float3 hl = hlf_of(cube);
    float4 hz = hit_zplane(hl.z, p, d);
    float4 hx = hit_xplane(hl.x, p, d);
    float4 hy = hit_yplane(hl.y, p, d);
    bool vz = hz.w > 0.0f && in_zface(hz, cube, cb);
    bool vx = hx.w > 0.0f && in_xface(hx, cube, cb);
    bool vy = hy.w > 0.0f && in_yface(hy, cube, cb);

    // candidates in the shader's fill order: entry, z, x, y
    float4 h[4];
    int sr[4];
    h[0] = e;
    sr[0] = 0;
    h[1] = h[2] = h[3] = e;
    sr[1] = sr[2] = sr[3] = 0;
    int hc = 1;
    if (vz) {
      h[1] = hz;
      sr[1] = 1;
      hc = 2;
    }
    if (vx) {
      if (hc == 1) {
        h[1] = hx;
        sr[1] = 2;
      } else {
        h[2] = hx;
        sr[2] = 2;
      }
      ++hc;
    }
    if (vy) {
      if (hc == 1) {
        h[1] = hy;
        sr[1] = 3;
      } else if (hc == 2) {
        h[2] = hy;
        sr[2] = 3;
      } else {
        h[3] = hy;
        sr[3] = 3;
      }
      ++hc;
    }

    // ordering by swaps, exactly as the shader's nested loop (:276-290)
#pragma unroll
    for (int i = 0; i < 3; ++i) {
#pragma unroll
      for (int j = i + 1; j < 4; ++j) {
        if (j < hc && h[j].w < h[i].w) {
          float4 t = h[i];
          h[i] = h[j];
          h[j] = t;
          int u = sr[i];
          sr[i] = sr[j];
          sr[j] = u;
        }
      }
    }

    // occupied octets: a child in either tree (:313-317)
    uint32_t occ = 0;
#pragma unroll
    for (int o = 0; o < 8; ++o)
      if (pick8(s0, s1, o) > 0 || pick8(d0, d1, o) > 0) occ |= 1u << o;

    uint32_t list = 0;
    int len = 0;
    int pre = -1;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      if (i < hc) {
        float4 ac = h[i];
        int oct = 0;
        if (ac.x > hl.x) oct = 1;
        if (ac.y < hl.y) oct += 2;
        if (ac.z < hl.z) oct += 4;
        if (oct == pre) {
          if (ac.x == hl.x)
            oct ^= 1;  // horpairs
          else if (ac.y == hl.y)
            oct ^= 2;  // verpairs
          else if (ac.z == hl.z)
            oct ^= 4;  // deppairs
        }
        pre = oct;
        if ((occ >> oct) & 1u) {
          list |= (uint32_t)(oct | (sr[i] << 3)) << (5 * len);
          ++len;
        }
      }
    }

    if (len > 0) {
      // descend into the nearest candidate (:334-367)
      int oct = list & 7;
      int src = (list >> 3) & 3;
      float4 isp = src == 0 ? e : (src == 1 ? hz : (src == 2 ? hx : hy));
      st.at(level, 0) = list | ((uint32_t)len << 20) | (1u << 23);
      st.at(level, 1) = (uint32_t)ns;
      st.at(level, 2) = (uint32_t)nd;
      if (++pushes > kMaxPushes) {
        r.oob = true;
        return;
      }
      ns = pick8(s0, s1, oct);
      nd = pick8(d0, d1, oct);
      cube = child_cube(cube, oct);
      e = isp;
      ++level;
      continue;
    }

    // ---- pop until a level has candidates left (:368-375) ----
    for (;;) {
      if (level == 0) {
        r.status = kMiss;
        r.oob = oob;
        return;
      }
      --level;
      uint32_t pk = st.at(level, 0);
      int nx = list_next(pk);
      if (EXACT) cube = parent_cube(cube, list_entry(pk, nx - 1) & 7);
      if (nx < list_len(pk)) {
        int c = list_entry(pk, nx);
        int oct = c & 7, src = c >> 3;
        float4 isp;
        if (!EXACT || src == 0) {
          float4 ecube, elev;
          replay(st, level, bc, e0, p, d, ecube, elev);
          cube = ecube;
          isp = elev;
        }
        if (src != 0) isp = plane_point(src, cube, p, d);
        if (++pushes > kMaxPushes) {
          r.oob = true;
          return;
        }
        st.at(level, 0) = (pk & ~(7u << 23)) | ((uint32_t)(nx + 1) << 23);
        int32_t ps = (int32_t)st.at(level, 1);
        int32_t pd = (int32_t)st.at(level, 2);
        ns = load_child(sc.tree[0], ps, level, oct, oob);
        nd = load_child(sc.tree[1], pd, level, oct, oob);
        cube = child_cube(cube, oct);
        e = isp;
        ++level;
        break;
      }
    }
  }
}

}  // namespace qbc
