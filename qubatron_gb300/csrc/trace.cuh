// Building blocks of the device traversal of qubatron's sparse octree (the
// joint static + dynamic `cube_trace_line` of
// src/qubatron/shaders/octree_fsh.c:138-379); walker.cuh assembles them.
//
// Results are bit-identical to the shader's FP32 arithmetic: this file must be
// compiled with -fmad=false (no fused multiply-add), IEEE division and sqrt and
// no flush-to-zero, and every expression keeps the shader's operation order.
// The only explicit FMAs are those of div_by_recip, an exact division.
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
// level is computed from the path bits when every cube coordinate is
// representable (checked on the host, EXACT = true; see walker.cuh), or else
// replayed from the root along the path.
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
  int32_t n;             // nodes held; index >= n reads as 0 and is reported
  int32_t box_depth;     // depth the leaf boxes were built for (boxes usable when maxlevel >= it)
  const uint32_t* cbox;  // per node, 16 words: its children's leaf boxes (boxes.cu); null: none
};

struct DevModel {
  const float4* col;  // (r, g, b, 1) per point, as an RGB32F texel reads
  const float4* nrm;  // (x, y, z, 1)
  int32_t n;
};

struct DevScene {
  DevTree tree[2];    // 0 static, 1 dynamic
  DevModel model[2];
  unsigned long long* box_words;  // when set: add the leaf-box words the walks read
};

enum : int { kMiss = 0, kLeaf = 1, kDiscard = 2 };


// ---- is_cube_{x,y,z}plane (octree_fsh.c:62-99), branch-free ----
// A ray parallel to the plane gets FLT_MAX in every component, as in the
// shader; the division then runs on a dummy divisor of 1 and its result is
// replaced, so any other ray gets exactly (c - p) / d and p + d * t.
__device__ __forceinline__ float4 hit_xplane(float x, float3 p, float3 d) {
  const bool par = d.x == 0.0f;
  const float w = (x - p.x) / (par ? 1.0f : d.x);
  return make_float4(par ? kFltMax : x, par ? kFltMax : p.y + d.y * w, par ? kFltMax : p.z + d.z * w,
                     par ? kFltMax : w);
}
__device__ __forceinline__ float4 hit_yplane(float y, float3 p, float3 d) {
  const bool par = d.y == 0.0f;
  const float w = (y - p.y) / (par ? 1.0f : d.y);
  return make_float4(par ? kFltMax : p.x + d.x * w, par ? kFltMax : y, par ? kFltMax : p.z + d.z * w,
                     par ? kFltMax : w);
}
__device__ __forceinline__ float4 hit_zplane(float z, float3 p, float3 d) {
  const bool par = d.z == 0.0f;
  const float w = (z - p.z) / (par ? 1.0f : d.z);
  return make_float4(par ? kFltMax : p.x + d.x * w, par ? kFltMax : p.y + d.y * w, par ? kFltMax : z,
                     par ? kFltMax : w);
}

// Correctly rounded a / b from y = RN(1 / b), by Markstein's method (P.
// Markstein, "Computation of elementary functions on the IBM RISC System/6000
// processor", IBM J. Res. Develop. 34(1), 1990; proofs in M. Cornea-Hasegan,
// R. Golliver, P. Markstein, "Correctness proofs outline for Newton-Raphson
// based floating-point divide and square root algorithms", ARITH 14, 1999):
// if y is within half an ulp of 1/b and q within one ulp of a/b, the
// remainder r = a - b q is exact in one FMA and RN(q + r y) = RN(a / b).
// q0 = RN(a y) is within 1.5 ulp, the first correction brings it within one
// ulp, the second rounds correctly. Valid when nothing overflows or
// underflows; callers use it only for rays whose magnitudes rule that out
// (recip_div_ok), and a test checks it against IEEE division.
__device__ __forceinline__ float div_by_recip(float a, float b, float y) {
  float q = __fmul_rn(a, y);
  float r = __fmaf_rn(-b, q, a);
  q = __fmaf_rn(r, y, q);
  r = __fmaf_rn(-b, q, a);
  return __fmaf_rn(r, y, q);
}

// Whether div_by_recip is exact for every plane hit of a ray from p along d
// in the basecube (0, S, S, S): numerators c - p with c a cube coordinate
// (0 or S on the basecube faces) or a midpoint in (0, S) are 0 or within
// [2^-62, 2^65] in magnitude when every |p| component is 0 or in
// [2^-62, 2^64] and S in [2^-20, 2^40]; with |d| components 0 or in
// [2^-40, 2^40] every quotient and remainder then stays normal. A zero
// direction component is fine (that plane is never hit).
__device__ __forceinline__ bool recip_div_ok(float3 p, float3 d, float S) {
  auto dir_ok = [](float v) {
    const float a = fabsf(v);
    return (a == 0.0f) | ((a >= 9.094947e-13f) & (a <= 1.0995116e12f));  // 2^-40 .. 2^40
  };
  auto pos_ok = [](float v) {
    const float a = fabsf(v);
    return (a == 0.0f) | ((a >= 2.1684043e-19f) & (a <= 1.8446744e19f));  // 2^-62 .. 2^64
  };
  return dir_ok(d.x) & dir_ok(d.y) & dir_ok(d.z) & pos_ok(p.x) & pos_ok(p.y) & pos_ok(p.z) &
         (S >= 9.536743e-07f) & (S <= 1.0995116e12f);  // 2^-20 .. 2^40
}

// The same plane hits without the parallel-ray sentinel: for a ray parallel
// to the plane the values are meaningless and the caller must treat the hit
// as invalid (the sentinel only ever makes the face test fail). Non-parallel
// rays get exactly the values above.
__device__ __forceinline__ float4 hit_xplane_raw(float x, float3 p, float3 d) {
  const float w = (x - p.x) / (d.x == 0.0f ? 1.0f : d.x);
  return make_float4(x, p.y + d.y * w, p.z + d.z * w, w);
}
__device__ __forceinline__ float4 hit_yplane_raw(float y, float3 p, float3 d) {
  const float w = (y - p.y) / (d.y == 0.0f ? 1.0f : d.y);
  return make_float4(p.x + d.x * w, y, p.z + d.z * w, w);
}
__device__ __forceinline__ float4 hit_zplane_raw(float z, float3 p, float3 d) {
  const float w = (z - p.z) / (d.z == 0.0f ? 1.0f : d.z);
  return make_float4(p.x + d.x * w, p.y + d.y * w, z, w);
}

// Plane hits with the division by reciprocal (rays where recip_div_ok).
__device__ __forceinline__ float4 hit_xplane_rcp(float x, float3 p, float3 d, float y) {
  const float w = div_by_recip(x - p.x, d.x, y);
  return make_float4(x, p.y + d.y * w, p.z + d.z * w, w);
}
__device__ __forceinline__ float4 hit_yplane_rcp(float yv, float3 p, float3 d, float y) {
  const float w = div_by_recip(yv - p.y, d.y, y);
  return make_float4(p.x + d.x * w, yv, p.z + d.z * w, w);
}
__device__ __forceinline__ float4 hit_zplane_rcp(float z, float3 p, float3 d, float y) {
  const float w = div_by_recip(z - p.z, d.z, y);
  return make_float4(p.x + d.x * w, p.y + d.y * w, z, w);
}

// Half-open face tests (octree_fsh.c:166-192, 263-271), evaluated without
// short-circuit branches.
__device__ __forceinline__ bool in_zface(float4 a, float4 t, float4 b) {
  return (t.x < a.x) & (a.x <= b.x) & (t.y > a.y) & (a.y >= b.y);
}
__device__ __forceinline__ bool in_xface(float4 a, float4 t, float4 b) {
  return (t.y > a.y) & (a.y >= b.y) & (t.z > a.z) & (a.z >= b.z);
}
__device__ __forceinline__ bool in_yface(float4 a, float4 t, float4 b) {
  return (t.x < a.x) & (a.x <= b.x) & (t.z > a.z) & (a.z >= b.z);
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
// Point of candidate source src (1 z, 2 x, 3 y bisecting plane) of cube t:
// hit_{z,x,y}plane of the cube's midpoint, as one plane hit whose axis is
// picked by selects (the same operations on the same operands, so the same
// bits), because lanes of a warp pop to candidates of different sources.
__device__ __forceinline__ float4 plane_point(int src, float4 t, float3 p, float3 d) {
  const float3 h = hlf_of(t);
  const bool ax = src == 2, ay = src == 3;
  const float c = ax ? h.x : (ay ? h.y : h.z);
  const float pa = ax ? p.x : (ay ? p.y : p.z);
  const float da = ax ? d.x : (ay ? d.y : d.z);
  const bool par = da == 0.0f;
  const float w = (c - pa) / (par ? 1.0f : da);
  const float x = ax ? c : p.x + d.x * w;
  const float y = ay ? c : p.y + d.y * w;
  const float z = (ax | ay) ? p.z + d.z * w : c;
  return make_float4(par ? kFltMax : x, par ? kFltMax : y, par ? kFltMax : z, par ? kFltMax : w);
}

// plane_point with the division by reciprocal (a valid candidate: its ray is
// not parallel to the plane). yr = RN(1 / d) per component.
__device__ __forceinline__ float4 plane_point_rcp(int src, float4 t, float3 p, float3 d, float3 yr) {
  const float3 h = hlf_of(t);
  const bool ax = src == 2, ay = src == 3;
  const float c = ax ? h.x : (ay ? h.y : h.z);
  const float pa = ax ? p.x : (ay ? p.y : p.z);
  const float da = ax ? d.x : (ay ? d.y : d.z);
  const float ya = ax ? yr.x : (ay ? yr.y : yr.z);
  const float w = div_by_recip(c - pa, da, ya);
  const float x = ax ? c : p.x + d.x * w;
  const float y = ay ? c : p.y + d.y * w;
  const float z = (ax | ay) ? p.z + d.z * w : c;
  return make_float4(x, y, z, w);
}

__device__ __forceinline__ int32_t pick8(int4 a, int4 b, int o) {
  int32_t lo = (o & 2) ? ((o & 1) ? a.w : a.z) : ((o & 1) ? a.y : a.x);
  int32_t hi = (o & 2) ? ((o & 1) ? b.w : b.z) : ((o & 1) ? b.y : b.x);
  return (o & 4) ? hi : lo;
}

// Child block of node i (oct_from_octets_for_index, octree_fsh.c:127-136):
// node 0 below the root is "no node"; a tree never uploaded holds nothing; an
// index outside the array reads as empty and is reported. One unsigned
// compare covers negative and too-large indices.
__device__ __forceinline__ bool load_block(const DevTree& t, int32_t i, int level, int4& a, int4& b,
                                           bool& oob) {
  const bool none = ((i == 0) & (level > 0)) | (t.n == 0);
  const bool bad = !none & ((uint32_t)i >= (uint32_t)t.n);
  oob |= bad;
  a = make_int4(0, 0, 0, 0);
  b = a;
  if (!none & !bad) {
    a = __ldg(t.child + 2 * (uint32_t)i);
    b = __ldg(t.child + 2 * (uint32_t)i + 1);
    return true;
  }
  return false;
}

__device__ __forceinline__ int32_t load_child(const DevTree& t, int32_t i, int level, int o, bool& oob) {
  const bool none = ((i == 0) & (level > 0)) | (t.n == 0);
  const bool bad = !none & ((uint32_t)i >= (uint32_t)t.n);
  oob |= bad;
  if (none | bad) return 0;
  return __ldg(reinterpret_cast<const int32_t*>(t.child) + 8 * (uint32_t)i + o);
}

__device__ __forceinline__ int32_t load_model(const DevTree& t, int32_t i, int level, bool& oob) {
  const bool none = ((i == 0) & (level > 0)) | (t.n == 0);
  const bool bad = !none & ((uint32_t)i >= (uint32_t)t.n);
  oob |= bad;
  if (none | bad) return 0;
  return __ldg(t.model + (uint32_t)i);
}

__device__ __forceinline__ void load_attr(const DevModel& m, int32_t i, float4& col, float4& nrm, bool& oob) {
  col = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  nrm = col;
  if (m.n == 0) return;
  if ((uint32_t)i >= (uint32_t)m.n) {
    oob = true;
    return;
  }
  col = __ldg(m.col + (uint32_t)i);
  nrm = __ldg(m.nrm + (uint32_t)i);
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


// Record word of child o in a node's leaf-box record (boxes.cu).
__device__ __forceinline__ uint2 child_box_word(const uint32_t* rec, int o) {
  return __ldg(reinterpret_cast<const uint2*>(rec) + o);
}

// Whether the ray p + t d (t >= 0) passes within m of the leaf box of a
// child. A miss proves that the walk finds no leaf below that child: every
// candidate point it computes lies within a small multiple of the
// coordinates' ulp of the ray, far below m, and a leaf is only reached
// through a point inside it.
//
// BoxFrame holds what the test of all children of one node shares: per axis
// the ray's t at the node's x-min (y-max, z-max) face moved outward by -m
// (a0) and +m (a1) along that axis, and the change of t per box unit (1/256
// of a child's edge) into the cube (u; y and z count downward). A bound q
// units into the cube is then one FMA: a + q * u. Against the direct slab
// test this regroups (c + q * unit +- m - p) / d; the extra rounding is a
// few ulps of coordinates below 9 S (one ulp is at most 2^-19 S), far inside
// m = 2^-14 S.
struct BoxFrame {
  float a0[3], a1[3], u[3];
};
__device__ __forceinline__ BoxFrame box_frame(float4 cube, float3 p, float3 inv, float m) {
  const float unit = cube.w * 0.001953125f;  // 1/512 of the node's edge
  BoxFrame f;
  const float ax = (cube.x - p.x) * inv.x, mx = m * inv.x;
  const float ay = (cube.y - p.y) * inv.y, my = m * inv.y;
  const float az = (cube.z - p.z) * inv.z, mz = m * inv.z;
  f.a0[0] = ax - mx;
  f.a1[0] = ax + mx;
  f.u[0] = unit * inv.x;
  f.a0[1] = ay - my;
  f.a1[1] = ay + my;
  f.u[1] = -(unit * inv.y);
  f.a0[2] = az - mz;
  f.a1[2] = az + mz;
  f.u[2] = -(unit * inv.z);
  return f;
}

// Test of child o with its record word r (boxes.cu: bytes xlo xhi ylo yhi,
// then zlo zhi, in units from the child's x-min, y-max, z-max corner).
__device__ __forceinline__ bool child_box_hit(uint2 r, int o, const BoxFrame& f) {
  // byte k of w as a float: bits 0x4B0000kk are 2^23 + k; subtracting
  // 2^23 - c gives k + c exactly (c: the child's offset of 256 units in the
  // node, plus 1 for a high bound's far side)
  auto q = [](uint32_t w, uint32_t sel, float k) { return __uint_as_float(__byte_perm(w, 0x4B000000u, sel)) - k; };
  const float kx = (o & 1) ? 8388352.0f : 8388608.0f, ky = (o & 2) ? 8388352.0f : 8388608.0f,
              kz = (o & 4) ? 8388352.0f : 8388608.0f;
  const float xlo = q(r.x, 0x7540u, kx), xhi = q(r.x, 0x7541u, kx - 1.0f);
  const float ylo = q(r.x, 0x7542u, ky), yhi = q(r.x, 0x7543u, ky - 1.0f);
  const float zlo = q(r.y, 0x7540u, kz), zhi = q(r.y, 0x7541u, kz - 1.0f);
  // x: low bound - m, high bound + m; y and z run downward, so their high
  // bound is the low coordinate
  float t0 = __fmaf_rn(xlo, f.u[0], f.a0[0]), t1 = __fmaf_rn(xhi, f.u[0], f.a1[0]);
  float tn = fminf(t0, t1), tf = fmaxf(t0, t1);
  t0 = __fmaf_rn(yhi, f.u[1], f.a0[1]);
  t1 = __fmaf_rn(ylo, f.u[1], f.a1[1]);
  tn = fmaxf(tn, fminf(t0, t1));
  tf = fminf(tf, fmaxf(t0, t1));
  t0 = __fmaf_rn(zhi, f.u[2], f.a0[2]);
  t1 = __fmaf_rn(zlo, f.u[2], f.a1[2]);
  tn = fmaxf(tn, fminf(t0, t1));
  tf = fminf(tf, fmaxf(t0, t1));
  return (xlo < xhi) & (tn <= tf) & (tf >= 0.0f);  // xlo >= xhi + 1: a subtree without leaves
}

// Whether a ray may reach a leaf of tree t: false when every child of the
// root is empty or its leaf box (widened by 2^-14 of the basecube edge) is
// missed, the filter's own test at the root. The caller has established the
// filter's conditions for the ray (exact basecube, nonzero direction
// components, origin within 8 edges, boxes built for the render's depth);
// without a usable box one level below the root the answer is true.
__device__ __forceinline__ bool root_box_near(const DevTree& t, float4 bc, float3 p, float3 inv) {
  if (t.cbox == nullptr || t.box_depth <= 1 || t.n == 0) return true;
  const int4 r0 = __ldg(t.child), r1 = __ldg(t.child + 1);
  uint32_t occ = 0;
#pragma unroll
  for (int o = 0; o < 8; ++o) occ |= pick8(r0, r1, o) > 0 ? (1u << o) : 0u;
  if (occ == 0u) return false;
  const BoxFrame bf = box_frame(bc, p, inv, bc.w * 6.1035156e-05f);
  // occupied children only (a character fills one or two octants)
#pragma unroll 1
  for (; occ; occ &= occ - 1u) {
    const int o = __ffs((int)occ) - 1;
    if (child_box_hit(child_box_word(t.cbox, o), o, bf)) return true;
  }
  return false;
}

// The same test out of line (for a kernel that runs it once per ray start,
// away from its walk's hot code); the tree's fields by value.
static __device__ __noinline__ bool root_box_near_call(const int4* child, const uint32_t* cbox, int32_t box_depth,
                                                       int32_t n, float4 bc, float3 p, float3 inv) {
  DevTree t;
  t.child = child;
  t.cbox = cbox;
  t.box_depth = box_depth;
  t.n = n;
  t.model = nullptr;
  return root_box_near(t, bc, p, inv);
}

}  // namespace qbc
