// Resumable traversal of qubatron's sparse octree, one step per call.
//
// Walks the static and dynamic trees together exactly as `cube_trace_line`
// of src/qubatron/shaders/octree_fsh.c:138-379 does, but as a state machine:
// start() does the basecube entry; each step() does one subnode test and one
// descent (after popping as far as needed). A persistent kernel can then give
// a lane whose ray ended a new ray, instead of idling until the slowest ray
// of its warp ends.
//
// Same arithmetic contract as trace.cuh (FP32 in the shader's order,
// -fmad=false, IEEE division) and the same shared-memory stack encoding:
//   word 0  sorted candidate list, 4 x (octet | source << 3) in 5-bit fields,
//           length in bits 20-22, next index in bits 23-25;
//   word 1  the level's static node index;
//   word 2  the level's dynamic node index (only with a dynamic tree).
//
// With EXACT (every cube coordinate representable: basecube (0, S, S, S) and
// the odd part of S has at most 24 - maxlevel bits) the current cube is not
// kept as floats but as its path: X, Y, Z hold one bit per level (the octet's
// x, y, z shift bits, root first), so the cube of level L is exactly
// (X * u, S - Y * u, S - Z * u, u) with u = S / 2^L, the same values the
// shader's successive halvings and shifts produce. A bit mask `more` marks
// the levels whose candidate lists have unused entries, so a pop jumps to
// its level in constant time (highest set bit, shift the path right) instead
// of walking up level by level.
#pragma once

#include "trace.cuh"

namespace qbc {

enum : int { kRunning = 3 };

// Whether the leaf-box filter applies to an EXACT ray (fdiv: its plane hits
// divide by reciprocals): every direction component nonzero (finite
// reciprocals) and the origin within 8 basecube edges s (candidate points
// then stay within ~2^-17 s of the ray, far inside the 2^-14 s margin).
__device__ __forceinline__ bool box_ray_ok(float3 p, float3 d, float s, bool fdiv) {
  const float r8 = 8.0f * s;
  return fdiv & (d.x != 0.0f) & (d.y != 0.0f) & (d.z != 0.0f) & (fabsf(p.x) <= r8) & (fabsf(p.y) <= r8) &
         (fabsf(p.z) <= r8);
}

template <bool EXACT, bool DYN, bool PROP = false>
struct Walker {
  float3 p, d;   // ray origin and direction
  float3 inv;    // EXACT: RN(1 / d) per component (0 for a zero component)
  // EXACT: bit 0 plane hits divide by reciprocal (div_by_recip); bits 1, 2
  // the candidates of the static / dynamic tree are filtered by the
  // children's leaf boxes (child_box_hit)
  uint32_t mode;
  float4 e0;     // entry point of the basecube (!EXACT; EXACT recomputes it)
  float4 cube;   // current cube (tlf.xyz, edge); !EXACT only
  uint32_t X, Y, Z;  // EXACT: path shift bits of the current cube, one per level
  uint32_t more;     // EXACT: bit L set when level L's candidate list has unused entries
  float4 e;      // entry point of the current cube
  int level;
  int32_t ns, nd;
  int pushes;
  bool oob;
  uint32_t vis_s, vis_d;
  // proposal test (PROP only): while level < tdepth the walk goes straight
  // to the cell of path `target` (3 bits per level, root first) through the
  // candidate the plain walk would use; below it, pops stop at tdepth.
  uint32_t target;
  int tdepth;

  static constexpr int kWords = DYN ? 3 : 2;

  __device__ __forceinline__ uint32_t& slot(const Stack& st, int l, int k) const {
    return st.base[(kWords * l + k) * st.stride];
  }

  // Cube of the current level from the path (EXACT): exact products and
  // sums, so equal to the successive child shifts.
  __device__ __forceinline__ float4 cube_of_path(float4 bc) const {
    const float u = bc.w * __int_as_float((127 - level) << 23);  // S / 2^level
    return make_float4(bc.x + (float)X * u, bc.y - (float)Y * u, bc.z - (float)Z * u, u);
  }

  // Basecube entry point (octree_fsh.c:157-211): false for a discard.
  __device__ __forceinline__ bool entry(float4 bc, float4& h0) const {
    float4 cb = brb_of(bc);
    int hitc = 0;
    float4 h1 = make_float4(0.f, 0.f, 0.f, 0.f), a;
    h0 = h1;
#define QB_FACE(expr, test)     \
  a = expr;                     \
  if (test) {                   \
    if (hitc == 0) h0 = a;      \
    else if (hitc == 1) h1 = a; \
    ++hitc;                     \
  }
    QB_FACE(hit_zplane(bc.z, p, d), in_zface(a, bc, cb))  // front
    QB_FACE(hit_zplane(cb.z, p, d), in_zface(a, bc, cb))  // back
    QB_FACE(hit_xplane(bc.x, p, d), in_xface(a, bc, cb))  // left
    QB_FACE(hit_xplane(cb.x, p, d), in_xface(a, bc, cb))  // right
    QB_FACE(hit_yplane(bc.y, p, d), in_yface(a, bc, cb))  // top
    QB_FACE(hit_yplane(cb.y, p, d), in_yface(a, bc, cb))  // bottom
#undef QB_FACE
    if (hitc < 2 || (h0.w < 0.0f && h1.w < 0.0f)) return false;
    if (h1.w < h0.w) h0 = h1;
    if (h0.w < 0.0f) h0 = make_float4(p.x, p.y, p.z, 0.0f);
    return true;
  }

  // Start a ray: the basecube entry. Returns kDiscard or kRunning.
  __device__ __forceinline__ int start(float4 bc, float3 rp, float3 rd, const DevScene& sc, int maxlevel) {
    p = rp;
    d = rd;
    cube = bc;
    X = Y = Z = 0u;
    more = 0u;
    level = 0;
    ns = 0;
    nd = 0;
    pushes = 0;
    oob = false;
    vis_s = 0;
    vis_d = 0;
    target = 0;
    tdepth = 0;
    if (EXACT) {
      const bool fdiv = recip_div_ok(p, d, bc.w);
      // boxes: a ray the filter applies to, and boxes built for a depth the
      // render reaches
      const bool geo = box_ray_ok(p, d, bc.w, fdiv);
      const bool bs = geo & (sc.tree[0].cbox != nullptr) & (maxlevel >= sc.tree[0].box_depth);
      const bool bd = DYN & geo & (sc.tree[1].cbox != nullptr) & (maxlevel >= sc.tree[1].box_depth);
      mode = (fdiv ? 1u : 0u) | (bs ? 2u : 0u) | (bd ? 4u : 0u);
      inv = make_float3(d.x == 0.0f ? 0.0f : __frcp_rn(d.x), d.y == 0.0f ? 0.0f : __frcp_rn(d.y),
                        d.z == 0.0f ? 0.0f : __frcp_rn(d.z));
      // bit 3: the ray misses the leaf box of every child of the dynamic
      // root, so it can reach no dynamic leaf and the walk leaves the
      // dynamic tree alone (the same pixels; no dynamic visits)
      if (DYN && bd && !root_box_near(sc.tree[1], bc, p, inv)) mode |= 8u;
    }
    float4 h0;
    if (!entry(bc, h0)) return kDiscard;
    if (!EXACT) e0 = h0;
    e = h0;
    return kRunning;
  }

  // After start(): whether a two-tree walk of this ray reads the dynamic
  // tree, i.e. Walker<EXACT, true>::start would not give it mode bit 3.
  __device__ __forceinline__ bool walks_dynamic(const DevScene& sc, float4 bc, int maxlevel) const {
    if (!EXACT) return true;
    const DevTree& t = sc.tree[1];
    if (!box_ray_ok(p, d, bc.w, (mode & 1u) != 0u) || t.cbox == nullptr || maxlevel < t.box_depth) return true;
    return root_box_near_call(t.child, t.cbox, t.box_depth, t.n, bc, p, inv);
  }

  // Cube and entry point of level lv replayed from the root along the path.
  __device__ __forceinline__ void replay_to(const Stack& st, int lv, float4 bc, float4& c, float4& en) const {
    c = bc;
    if (EXACT)
      entry(bc, en);  // the ray was entered, so this succeeds
    else
      en = e0;
    for (int k = 0; k < lv; ++k) {
      uint32_t pk = slot(st, k, 0);
      int cc = list_entry(pk, list_next(pk) - 1);
      if (cc >> 3) en = plane_point(cc >> 3, c, p, d);
      c = child_cube(c, cc & 7);
    }
  }

  // One step: the subnode test of the current (freshly entered) cube, then
  // either the descent into its nearest candidate or pops up to the nearest
  // level with candidates left and the descent into the next one there.
  // Every step of every lane thus runs exactly one subnode test, so the
  // lanes of a warp stay on the same instructions for the expensive part.
  // Returns kRunning, kLeaf (fields via leaf()) or kMiss.
  // `fast`: every lane of the warp that steps now may divide by its
  // reciprocals (a vote the caller takes when rays start).
  __device__ __forceinline__ int step(const DevScene& sc, int maxlevel, float4 bc, const Stack& st, bool fast) {
    if (level == maxlevel) return kLeaf;

    if (EXACT) cube = cube_of_path(bc);

    // ---- subnode test (octree_fsh.c:251-329) ----
    // dl: the ray walks the dynamic tree too (mode bit 3, set at the start)
    const bool dl = DYN && (!EXACT || !(mode & 8u));
    int4 s0, s1, d0 = make_int4(0, 0, 0, 0), d1 = d0;
    // with one tree a node below the root is always a child index > 0 (the
    // walk only enters occupied children), so the node-0 rule needs no test
    if (load_block(sc.tree[0], ns, DYN ? level : 0, s0, s1, oob)) ++vis_s;
    if (dl) {
      if (load_block(sc.tree[1], nd, level, d0, d1, oob)) ++vis_d;
    }
    float4 cb = brb_of(cube);
    float3 hl = hlf_of(cube);
    // a ray parallel to a bisecting plane has no hit on it (the shader's
    // FLT_MAX sentinel fails the face test). With the reciprocal the
    // parallel component's reciprocal is 0, so the hit's t is +-0 and fails
    // t > 0 by itself; the single-tree kernels skip the test there (the
    // two-tree ones keep one form, which needs fewer registers).
    float4 hz, hx, hy;
    bool vz, vx, vy;
    if (EXACT && !DYN && fast) {
      hz = hit_zplane_rcp(hl.z, p, d, inv.z);
      hx = hit_xplane_rcp(hl.x, p, d, inv.x);
      hy = hit_yplane_rcp(hl.y, p, d, inv.y);
      vz = (hz.w > 0.0f) & in_zface(hz, cube, cb);
      vx = (hx.w > 0.0f) & in_xface(hx, cube, cb);
      vy = (hy.w > 0.0f) & in_yface(hy, cube, cb);
    } else {
      if (EXACT && fast) {
        hz = hit_zplane_rcp(hl.z, p, d, inv.z);
        hx = hit_xplane_rcp(hl.x, p, d, inv.x);
        hy = hit_yplane_rcp(hl.y, p, d, inv.y);
      } else {
        hz = hit_zplane_raw(hl.z, p, d);
        hx = hit_xplane_raw(hl.x, p, d);
        hy = hit_yplane_raw(hl.y, p, d);
      }
      vz = (d.z != 0.0f) & (hz.w > 0.0f) & in_zface(hz, cube, cb);
      vx = (d.x != 0.0f) & (hx.w > 0.0f) & in_xface(hx, cube, cb);
      vy = (d.y != 0.0f) & (hy.w > 0.0f) & in_yface(hy, cube, cb);
    }

    // Candidates in the shader's fill order (entry, z, x, y) as (t, code):
    // code = octet side bits | source << 3 | flip << 5. A bisecting-plane
    // hit lies on its own plane (its coordinate is the midpoint itself), so
    // its side bit on that axis is 0. The shader compacts the valid hits
    // before ordering them; here an invalid hit keeps its slot with t = +inf.
    // A valid candidate has a finite t, and the swap network (swap when
    // strictly less) then yields the valid candidates first, in the same
    // order as from the compacted array, ties included (checked for every
    // validity pattern and every tie pattern of 3 and 4 values).
    //
    // flip is the octet bit the pair fix-up (:301-309) toggles when the point
    // falls in the same octet as the candidate before it: the first axis, x
    // then y then z, on which the point equals the midpoint. A plane hit
    // always equals it on its own axis, so an x hit flips x, a y hit x or
    // y, a z hit x, y or z; only the entry point may flip nothing. The
    // fix-up is common (a ray crossing a bisecting plane towards its high
    // side meets it), so the flips are found here, where the points are at
    // hand, instead of in a branch per candidate.
    const float kInf = __int_as_float(0x7f800000);
    float t[4];
    uint32_t c[4];
    t[0] = e.w;
    c[0] = (e.x > hl.x ? 1u : 0u) | (e.y < hl.y ? 2u : 0u) | (e.z < hl.z ? 4u : 0u) |
           (e.x == hl.x ? 1u << 5 : (e.y == hl.y ? 2u << 5 : (e.z == hl.z ? 4u << 5 : 0u)));
    {
      const uint32_t cz = (hz.x > hl.x ? 1u : 0u) | (hz.y < hl.y ? 2u : 0u) | (1u << 3) |
                          (hz.x == hl.x ? 1u << 5 : (hz.y == hl.y ? 2u << 5 : 4u << 5));
      const uint32_t cx = (hx.y < hl.y ? 2u : 0u) | (hx.z < hl.z ? 4u : 0u) | (2u << 3) | (1u << 5);
      const uint32_t cy = (hy.x > hl.x ? 1u : 0u) | (hy.z < hl.z ? 4u : 0u) | (3u << 3) |
                          (hy.x == hl.x ? 1u << 5 : 2u << 5);
      t[1] = vz ? hz.w : kInf;
      c[1] = cz;
      t[2] = vx ? hx.w : kInf;
      c[2] = cx;
      t[3] = vy ? hy.w : kInf;
      c[3] = cy;
    }
    const int hc = 1 + (int)vz + (int)vx + (int)vy;
    // ordering by swaps, as the shader's nested loop (:276-290). When no
    // plane hit's t is below the entry's (the rule, unless the entry lies on
    // a bisecting plane) the first pass swaps nothing and the passes left are
    // the same network on slots 1..3; the warp takes that path when all its
    // lanes can.
    auto order = [&](int i, int j) {
      if (t[j] < t[i]) {
        float tt = t[i];
        t[i] = t[j];
        t[j] = tt;
        uint32_t cc = c[i];
        c[i] = c[j];
        c[j] = cc;
      }
    };
    if (__all_sync(__activemask(), t[0] <= fminf(t[1], fminf(t[2], t[3])))) {
      order(1, 2);
      order(1, 3);
      order(2, 3);
    } else {
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = i + 1; j < 4; ++j) order(i, j);
    }
    // occupied octets: a child in either tree (:313-317)
    uint32_t occ_s = 0, occ_d = 0;
#pragma unroll
    for (int o = 0; o < 8; ++o) {
      occ_s |= pick8(s0, s1, o) > 0 ? (1u << o) : 0u;
      if (DYN) occ_d |= pick8(d0, d1, o) > 0 ? (1u << o) : 0u;
    }
    const uint32_t occ = occ_s | occ_d;
    // leaf boxes of the children (EXACT rays that allow them)
    // (not one level above the tree's deepest: a child there is a leaf
    // cell, its box the whole child cube, which every listed child meets)
    const bool box_s = EXACT && (mode & 2u) && level + 1 < sc.tree[0].box_depth;
    const bool box_d = EXACT && DYN && (mode & 4u) && level + 1 < sc.tree[1].box_depth;
    const bool boxes = box_s || box_d;
    const uint32_t* rec_s = box_s ? sc.tree[0].cbox + (size_t)(uint32_t)ns * 16 : nullptr;
    const uint32_t* rec_d = box_d ? sc.tree[1].cbox + (size_t)(uint32_t)nd * 16 : nullptr;
    uint32_t pk = 0;
    int len = 0, pre = -1;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      if (i < hc) {
        int oct = c[i] & 7;
        const uint32_t src = (c[i] >> 3) & 3u;
        if (oct == pre) oct ^= (int)(c[i] >> 5);  // pair fix-up
        pre = oct;
        if ((occ >> oct) & 1u) {
          pk |= (uint32_t)(oct | (src << 3)) << (5 * len);
          ++len;
        }
      }
    }
    if (boxes && len > 0) {
      // keep a candidate when a tree holding that child may have a leaf near
      // the ray
      if (sc.box_words) {
        // instrumented renders: the box words the filter reads
        uint32_t nw = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const uint32_t bit = 1u << ((pk >> (5 * k)) & 7u);
          if (k < len) nw += ((occ_s & bit) && rec_s ? 1u : 0u) + ((occ_d & bit) && rec_d ? 1u : 0u);
        }
        const unsigned m = __activemask();
        const unsigned tot = __reduce_add_sync(m, nw);
        if ((int)(threadIdx.x & 31u) == __ffs((int)m) - 1) atomicAdd(sc.box_words, (unsigned long long)tot);
      }
      const BoxFrame bf = box_frame(cube, p, inv, bc.w * 6.1035156e-05f);  // margin 2^-14 S
      uint32_t q = 0;
      int nl = 0;
      if constexpr (!DYN) {
        // the records of all listed children first (independent loads), then
        // the tests
        uint2 ws[4];
#pragma unroll
        for (int k = 0; k < 4; ++k)
          ws[k] = (k < len && rec_s) ? child_box_word(rec_s, (int)((pk >> (5 * k)) & 7u)) : make_uint2(0u, 0u);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          if (k < len) {
            const uint32_t e = (pk >> (5 * k)) & 31u;
            const int oct = (int)(e & 7u);
            if (!rec_s || child_box_hit(ws[k], oct, bf)) {
              q |= e << (5 * nl);
              ++nl;
            }
          }
        }
      } else {
        // two trees: one child at a time keeps the registers in bounds
#pragma unroll 1
        for (int k = 0; k < len; ++k) {
          const uint32_t e = (pk >> (5 * k)) & 31u;
          const int oct = (int)(e & 7u);
          const bool hs = ((occ_s >> oct) & 1u) &&
                          (!rec_s || child_box_hit(child_box_word(rec_s, oct), oct, bf));
          const bool hd = ((occ_d >> oct) & 1u) &&
                          (!rec_d || child_box_hit(child_box_word(rec_d, oct), oct, bf));
          if (hs | hd) {
            q |= e << (5 * nl);
            ++nl;
          }
        }
      }
      pk = q;
      len = nl;
    }
    pk |= (uint32_t)len << 20;

    int nx = 0;
    if (PROP && level < tdepth) {
      // directed descent: the first candidate into the target's octet; if
      // there is none, the plain walk never enters the target cell here
      const int want = (int)(target >> (3 * (tdepth - 1 - level))) & 7;
      nx = -1;
#pragma unroll
      for (int k = 3; k >= 0; --k)
        if (k < len && (list_entry(pk, k) & 7) == want) nx = k;
      if (nx < 0) return kMiss;
    }
    float4 isp;
    int32_t cs, cd = 0;
    int cc;
    if constexpr (EXACT) {
      // ---- descend (:334-367) or pop (:368-375), as one sequence ----
      // A descent is a pop of no levels whose list and parent node are the
      // current ones; the lanes of a warp then follow one path. A pop jumps
      // to the nearest level above with unused candidates.
      const bool pop = len == 0;
      const uint32_t m = PROP ? (more & ~((1u << tdepth) - 1u)) : more;
      if (pop && m == 0u) return kMiss;
      const int lv = pop ? 31 - __clz(m) : level;
      const int up = level - lv;
      X >>= up;
      Y >>= up;
      Z >>= up;
      level = lv;
      const uint32_t saved = slot(st, level, 0);
      const int32_t parent = pop ? (int32_t)slot(st, level, 1) : ns;
      int32_t parent_d = 0;
      if (DYN) parent_d = pop ? (int32_t)slot(st, level, 2) : nd;
      pk = pop ? saved : pk;
      nx = pop ? list_next(pk) : nx;
      if (pop) cube = cube_of_path(bc);
      cc = list_entry(pk, nx);
      isp = e;
      if (pop && (cc >> 3) == 0) {
        float4 rc, re;
        replay_to(st, level, bc, rc, re);
        cube = rc;
        isp = re;
      }
      // the child is read again (an L1 hit) rather than kept from the
      // node's block: 6 blocks per SM fit in the registers. With one tree
      // the parent is a node whose block was read (a candidate exists only
      // below an occupied octet), so the index needs no checks.
      if (DYN)
        cs = load_child(sc.tree[0], parent, level, cc & 7, oob);
      else
        cs = __ldg(reinterpret_cast<const int32_t*>(sc.tree[0].child) + 8 * (uint32_t)parent + (cc & 7));
      slot(st, level, 1) = (uint32_t)parent;
      if (DYN) {
        cd = dl ? load_child(sc.tree[1], parent_d, level, cc & 7, oob) : 0;
        slot(st, level, 2) = (uint32_t)parent_d;
      }
    } else if (len > 0) {
      // ---- descend into the nearest candidate (:334-367) ----
      // (a plane hit is recomputed below from its source, with the same
      // operations: cheaper than keeping all three live through the filter)
      cc = PROP ? list_entry(pk, nx) : (int)(pk & 31);
      isp = e;
      cs = pick8(s0, s1, cc & 7);
      if (DYN) cd = pick8(d0, d1, cc & 7);
      slot(st, level, 1) = (uint32_t)ns;
      if (DYN) slot(st, level, 2) = (uint32_t)nd;
    } else {
      // ---- pop until a level has candidates left (:368-375) ----
      if (EXACT) {
        // the nearest level above with unused candidates, in one jump
        const uint32_t m = PROP ? (more & ~((1u << tdepth) - 1u)) : more;
        if (m == 0u) return kMiss;
        const int lv = 31 - __clz(m);
        const int up = level - lv;
        X >>= up;
        Y >>= up;
        Z >>= up;
        level = lv;
        pk = slot(st, level, 0);
        nx = list_next(pk);
        cube = cube_of_path(bc);
      } else {
        for (;;) {
          if (level == (PROP ? tdepth : 0)) return kMiss;
          --level;
          pk = slot(st, level, 0);
          nx = list_next(pk);
          if (nx < list_len(pk)) break;
        }
      }
      cc = list_entry(pk, nx);
      if (!EXACT || (cc >> 3) == 0) {
        float4 rc, re;
        replay_to(st, level, bc, rc, re);
        cube = rc;
        isp = re;
      }
      int32_t ps = (int32_t)slot(st, level, 1);
      cs = load_child(sc.tree[0], ps, level, cc & 7, oob);
      if (DYN) {
        int32_t pd = (int32_t)slot(st, level, 2);
        cd = load_child(sc.tree[1], pd, level, cc & 7, oob);
      }
    }
    {
      const int src = cc >> 3;
      if (src != 0) {
        if (EXACT && fast)
          isp = plane_point_rcp(src, cube, p, d, inv);
        else
          isp = plane_point(src, cube, p, d);
      }
    }
    if (++pushes > kMaxPushes) {
      oob = true;
      return kMiss;
    }
    slot(st, level, 0) = (pk & ~(7u << 23)) | ((uint32_t)(nx + 1) << 23);
    if (EXACT) {
      more = (more & ~(1u << level)) | (nx + 1 < list_len(pk) ? (1u << level) : 0u);
      X = (X << 1) | (uint32_t)(cc & 1);
      Y = (Y << 1) | (uint32_t)((cc >> 1) & 1);
      Z = (Z << 1) | (uint32_t)((cc >> 2) & 1);
    } else {
      cube = child_cube(cube, cc & 7);
    }
    e = isp;
    ns = cs;
    nd = cd;
    ++level;
    // a descent into the last level is the leaf hit (the loop's next pass
    // would return it before any subnode test, octree_fsh.c:218)
    return level == maxlevel ? kLeaf : kRunning;
  }

  // Leaf fetch (octree_fsh.c:218-247); call after step() returned kLeaf.
  __device__ __forceinline__ void leaf(const DevScene& sc, int32_t& ms, int32_t& md, float4& col, float4& nrm) {
    ms = load_model(sc.tree[0], ns, level, oob);
    md = DYN ? load_model(sc.tree[1], nd, level, oob) : 0;
    load_attr(sc.model[0], ms, col, nrm, oob);
    if (DYN && md > 0) load_attr(sc.model[1], md, col, nrm, oob);
  }
};


}  // namespace qbc
