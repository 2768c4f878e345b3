// GPU node-array builder: the same node array as inserting points one by one
// with octree_insert_point (src/qubatron/octree.c:95-147) or octet paths with
// octree_insert_path (octree.c:149-180) into an empty tree, numbering
// included, without the sequential walk, without sorting and without any host
// round trip, so that a per-frame rebuild can be captured in a CUDA graph.
//
// Sequential insertion appends a node the first time a path prefix appears:
// point i walks down the nodes earlier points made and appends the rest of
// its path. So the node of a level-l prefix is created by the smallest point
// index having that prefix (its "creator"), and point i creates exactly the
// levels [c_i, levels] where c_i is the first level whose node it creates.
// Node ids follow from one prefix sum over points in index order:
//   id(i, l) = 1 + sum_{j < i} (levels - c_j + 1) + (l - c_i).
//
// Creators, level by level, with one kernel per level: the level-l group of
// a point is (creator of its level-(l-1) node, its level-l octet), a slot
// creator * 8 + octet of a table the points atomicMin their index into; the
// next kernel reads the winner. Warps merge equal slots first (their lanes'
// indices increase, so the lowest lane of a group holds its minimum). The
// top levels, whose few groups every block meets, use tables indexed by the
// prefix itself, reduced in shared memory per block first. The deeper
// levels rotate three tables of 8 entries per point; a table's entries are
// reset to "empty" by the kernel two levels later, so the tables are empty
// again when the build ends.
//
// Leaf boxes come from the same per-point enumeration of the nodes (the
// creator of a level-l node visits it): bottom up, each node's box of leaf
// cells is the union of its children's, and its record holds its children's
// boxes quantised outward to 1/256 of a child's edge, the format the render
// kernels' pruning reads (boxes.cu builds the same records for uploaded
// trees).

#include <cuda_runtime.h>
#include <thrust/device_vector.h>
#include <thrust/execution_policy.h>
#include <thrust/sort.h>

#include <cstdint>
#include <vector>

#include "qbc_internal.h"
#include "qbcuda.h"

using qbc::fail;

namespace qbc {
namespace {

constexpr int kMaxBuildLevels = 21;   // 3 bits per level in a 64-bit key
constexpr int kDense = 4;             // levels 1..kDense use prefix-indexed tables
constexpr int kDenseEntries = 8 + 64 + 512 + 4096;
constexpr uint64_t kExcluded = ~0ull;  // key of a point left out (bad input)
constexpr uint32_t kNone = 0xFFFFFFFFu;
constexpr int kScanThreads = 256, kScanPer = 8, kScanChunk = kScanThreads * kScanPer;

__host__ __device__ constexpr int dense_offset(int l) {  // first entry of level l's prefix table
  return l <= 1 ? 0 : (l == 2 ? 8 : (l == 3 ? 72 : 584));
}

// Path keys (octets of octree.c:100-109 for points: size halves from the
// basecube edge, (int)(x / size) % 2 picks the x bit, y and z below the
// midline set bits 1 and 2; or the given octets), and the per-point state.
__global__ void keys_kernel(const float* __restrict__ pts, const int32_t* __restrict__ octets, int64_t n,
                            float basesize, int levels, uint64_t* __restrict__ key, uint8_t* __restrict__ own,
                            uint32_t* __restrict__ cre, uint32_t* __restrict__ slot, uint32_t* __restrict__ slot_old,
                            uint32_t* __restrict__ par, unsigned* __restrict__ err) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    uint64_t k = 0;
    bool ok = true;
    if (pts) {
      const float x = pts[3 * i], y = pts[3 * i + 1], z = pts[3 * i + 2];
      if (!(x >= 0.0f && x < 1.0e30f && y >= 0.0f && y < 1.0e30f && z >= 0.0f && z < 1.0e30f)) {
        ok = false;
      } else {
        float size = basesize;
        for (int level = 0; level < levels; ++level) {
          size /= 2.0f;
          int octet = (int)(x / size) % 2;
          int yi = (int)(y / size) % 2;
          int zi = (int)(z / size) % 2;
          if (yi == 0) octet += 2;
          if (zi == 0) octet += 4;
          k = (k << 3) | (uint64_t)octet;
        }
      }
    } else {
      for (int level = 0; level < levels; ++level) {
        const int o = octets[i * levels + level];
        ok = ok && o >= 0 && o <= 7;
        k = (k << 3) | (uint64_t)(o & 7);
      }
    }
    if (!ok) atomicOr(err, pts ? kErrBuildPoint : kErrBuildOctet);
    key[i] = ok ? k : kExcluded;
    own[i] = (uint8_t)(levels + 1);
    cre[i] = kNone;  // the root
    slot[i] = kNone;
    slot_old[i] = kNone;
    par[i] = kNone;
  }
}

// Level l: resolve level l - 1 (read the creator of the point's group, note
// the first level the point creates), reset the level l - 2 table entries,
// and propose level l (atomicMin of the point index into its group's slot).
// l runs 1..levels + 1; the last call only resolves.
__global__ void level_kernel(int l, int levels, int64_t n, const uint64_t* __restrict__ key,
                             uint8_t* __restrict__ own, uint32_t* __restrict__ cre, uint32_t* __restrict__ slot,
                             uint32_t* __restrict__ slot_old, uint32_t* __restrict__ par,
                             const uint32_t* __restrict__ t_res, uint32_t* __restrict__ t_clr,
                             uint32_t* __restrict__ t_prop, int prop_dense) {
  extern __shared__ uint32_t sm[];
  const int entries = prop_dense ? (1 << (3 * l)) : 0;
  for (int e = threadIdx.x; e < entries; e += blockDim.x) sm[e] = kNone;
  if (prop_dense) __syncthreads();
  const int lane = threadIdx.x & 31;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t b0 = (int64_t)blockIdx.x * blockDim.x; b0 < n; b0 += stride) {  // same trip count per block
    const int64_t i = b0 + threadIdx.x;
    const bool valid = i < n && key[i] != kExcluded;
    uint32_t s = kNone;
    if (valid) {
      uint64_t k = key[i];
      uint32_t c = cre[i];
      uint32_t so = slot[i];
      if (l >= 2) {
        const uint32_t w = t_res[so];
        if (w == (uint32_t)i && own[i] == (uint8_t)(levels + 1)) {
          own[i] = (uint8_t)(l - 1);
          par[i] = c;
        }
        c = w;
        cre[i] = c;
        if (t_clr) {
          const uint32_t sc = slot_old[i];
          if (sc != kNone) t_clr[sc] = kNone;
        }
      }
      if (l <= levels) {
        const uint64_t prefix = k >> (3 * (levels - l));
        s = prop_dense ? (uint32_t)prefix : c * 8u + (uint32_t)(prefix & 7u);
        slot_old[i] = so;
        slot[i] = s;
      }
    }
    if (l <= levels) {
      if (prop_dense) {
        if (valid) atomicMin(&sm[s], (uint32_t)i);
      } else {
        const unsigned group = __match_any_sync(0xFFFFFFFFu, s);
        if (valid && lane == __ffs(group) - 1) atomicMin(&t_prop[s], (uint32_t)i);
      }
    }
  }
  if (prop_dense) {
    __syncthreads();
    for (int e = threadIdx.x; e < entries; e += blockDim.x)
      if (sm[e] != kNone) atomicMin(&t_prop[e], sm[e]);
  }
}

__device__ __forceinline__ int32_t made(const uint8_t* own, const uint64_t* key, int64_t i, int64_t n, int levels) {
  if (i >= n || key[i] == kExcluded) return 0;
  const int o = own[i];
  return o <= levels ? levels - o + 1 : 0;
}

// Prefix sum, pass 1: nodes made per chunk of kScanChunk points; also resets
// the last level's creator-table entries (all of that level's reads are done).
__global__ void scan_chunks_kernel(const uint8_t* __restrict__ own, const uint64_t* __restrict__ key, int64_t n,
                                   int levels, const uint32_t* __restrict__ slot, uint32_t* __restrict__ t_last,
                                   int32_t* __restrict__ blocksum) {
  __shared__ int32_t red[kScanThreads];
  const int64_t b = blockIdx.x;
  int32_t sum = 0;
  for (int k = 0; k < kScanPer; ++k) {
    const int64_t i = b * kScanChunk + (int64_t)threadIdx.x * kScanPer + k;
    sum += made(own, key, i, n, levels);
    if (t_last && i < n && key[i] != kExcluded) t_last[slot[i]] = kNone;
  }
  red[threadIdx.x] = sum;
  __syncthreads();
  for (int o = kScanThreads / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) blocksum[b] = red[0];
}

// Pass 2 (one block): exclusive scan of the chunk sums in place; the node
// count (with the root) to *total.
__global__ void scan_top_kernel(int32_t* __restrict__ blocksum, int64_t nb, int32_t* __restrict__ total) {
  __shared__ int32_t sh[1024];
  int32_t carry = 1;  // node 0 is the root
  for (int64_t b0 = 0; b0 < nb; b0 += 1024) {
    const int64_t b = b0 + threadIdx.x;
    const int32_t v = b < nb ? blocksum[b] : 0;
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
      const int32_t t = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
      __syncthreads();
      sh[threadIdx.x] += t;
      __syncthreads();
    }
    if (b < nb) blocksum[b] = carry + sh[threadIdx.x] - v;
    const int32_t add = sh[1023];
    __syncthreads();
    carry += add;
  }
  if (threadIdx.x == 0) *total = carry;
}

// Pass 3: each point's first node id; clear the child blocks of the nodes
// it makes, set their model indices, and give its leaf node the box of its
// own cell.
__global__ void scan_nodes_kernel(const uint8_t* __restrict__ own, const uint64_t* __restrict__ key, int64_t n,
                                  int levels, const int32_t* __restrict__ blocksum, int32_t* __restrict__ base,
                                  int64_t first_index, int4* __restrict__ child, int32_t* __restrict__ model,
                                  int32_t* __restrict__ box) {
  __shared__ int32_t sh[kScanThreads];
  const int64_t b = blockIdx.x;
  int32_t mine[kScanPer], sum = 0;
  for (int k = 0; k < kScanPer; ++k) {
    mine[k] = made(own, key, b * kScanChunk + (int64_t)threadIdx.x * kScanPer + k, n, levels);
    sum += mine[k];
  }
  sh[threadIdx.x] = sum;
  __syncthreads();
  for (int o = 1; o < kScanThreads; o <<= 1) {
    const int32_t t = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
    __syncthreads();
    sh[threadIdx.x] += t;
    __syncthreads();
  }
  int32_t id = blocksum[b] + sh[threadIdx.x] - sum;
  if (b == 0 && threadIdx.x == 0) {
    child[0] = make_int4(0, 0, 0, 0);
    child[1] = make_int4(0, 0, 0, 0);
    model[0] = 0;
  }
  for (int k = 0; k < kScanPer; ++k) {
    const int64_t i = b * kScanChunk + (int64_t)threadIdx.x * kScanPer + k;
    if (i >= n) break;
    base[i] = id;
    for (int m = 0; m < mine[k]; ++m) {
      child[2 * (int64_t)(id + m)] = make_int4(0, 0, 0, 0);
      child[2 * (int64_t)(id + m) + 1] = make_int4(0, 0, 0, 0);
      model[id + m] = (int32_t)(i + first_index);
    }
    if (mine[k] > 0) {
      int32_t* bx = box + (int64_t)(id + mine[k] - 1) * 6;
      bx[0] = bx[1] = bx[2] = bx[3] = bx[4] = bx[5] = 0;
    }
    id += mine[k];
  }
}

// Every made node links itself into its parent.
__global__ void link_kernel(const uint64_t* __restrict__ key, const uint8_t* __restrict__ own,
                            const uint32_t* __restrict__ par, const int32_t* __restrict__ base, int64_t n, int levels,
                            int32_t* __restrict__ child) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t k = key[i];
    const int o = own[i];
    if (k == kExcluded || o > levels) continue;
    const int32_t id0 = base[i];
    int32_t parent = 0;
    if (o > 1) {
      const uint32_t p = par[i];
      parent = base[p] + (o - 1 - own[p]);
    }
    for (int l = o; l <= levels; ++l) {
      const int32_t id = id0 + (l - o);
      const int oct = (int)((k >> (3 * (levels - l))) & 7u);
      child[(int64_t)parent * 8 + oct] = id;
      parent = id;
    }
  }
}

// Level l's nodes (l < levels): each node's leaf-cell box from its children's
// (children at level l + 1, done) and its record. The creator of a node
// visits it; the root is visited by thread 0 of the l = 0 launch.
__global__ void box_kernel(int l, int levels, const uint64_t* __restrict__ key, const uint8_t* __restrict__ own,
                           const int32_t* __restrict__ base, int64_t n, const int32_t* __restrict__ child,
                           int32_t* __restrict__ box, uint32_t* __restrict__ rec) {
  const int32_t child_cells = 1 << (levels - l - 1);  // leaf cells along a child's edge
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (l == 0 ? 1 : n); i += stride) {
    int32_t node;
    if (l == 0) {
      node = 0;
    } else {
      const int o = own[i];
      if (key[i] == kExcluded || o > l) continue;
      node = base[i] + (l - o);
    }
    int32_t r[6] = {0x7fffffff, -1, 0x7fffffff, -1, 0x7fffffff, -1};
    uint32_t w[16];
    const int4* cb4 = reinterpret_cast<const int4*>(child + (int64_t)node * 8);
    const int4 c0 = cb4[0], c1 = cb4[1];
    const int32_t ch[8] = {c0.x, c0.y, c0.z, c0.w, c1.x, c1.y, c1.z, c1.w};
#pragma unroll
    for (int o = 0; o < 8; ++o) {
      uint32_t q[6] = {255u, 0u, 255u, 0u, 255u, 0u};  // empty
      if (ch[o] > 0) {
        const int32_t* cb = box + (int64_t)ch[o] * 6;
        if (cb[0] <= cb[1]) {
          const int32_t off[3] = {(o & 1) ? child_cells : 0, (o & 2) ? child_cells : 0, (o & 4) ? child_cells : 0};
#pragma unroll
          for (int a = 0; a < 3; ++a) {
            r[2 * a] = min(r[2 * a], cb[2 * a] + off[a]);
            r[2 * a + 1] = max(r[2 * a + 1], cb[2 * a + 1] + off[a]);
            // [lo, hi + 1) leaf cells in 1/256 of the child's edge, rounded outward
            const int64_t lo = cb[2 * a], hi1 = (int64_t)cb[2 * a + 1] + 1;
            const int64_t ql = lo * 256 / child_cells;
            const int64_t qh = (hi1 * 256 + child_cells - 1) / child_cells - 1;
            q[2 * a] = (uint32_t)(ql < 0 ? 0 : (ql > 255 ? 255 : ql));
            q[2 * a + 1] = (uint32_t)(qh < 0 ? 0 : (qh > 255 ? 255 : qh));
          }
        }
      }
      w[2 * o] = q[0] | (q[1] << 8) | (q[2] << 16) | (q[3] << 24);
      w[2 * o + 1] = q[4] | (q[5] << 8);
    }
    int32_t* nb = box + (int64_t)node * 6;
#pragma unroll
    for (int a = 0; a < 6; ++a) nb[a] = r[a];
    uint4* dst = reinterpret_cast<uint4*>(rec + (int64_t)node * 16);
#pragma unroll
    for (int k = 0; k < 4; ++k) dst[k] = make_uint4(w[4 * k], w[4 * k + 1], w[4 * k + 2], w[4 * k + 3]);
  }
}

template <typename T>
int grow_buf(T** p, int64_t have, int64_t need, const char* what) {
  if (have >= need && *p) return QBC_OK;
  if (*p) cudaFree(*p);
  *p = nullptr;
  cudaError_t e = cudaMalloc((void**)p, (size_t)std::max<int64_t>(need, 1) * sizeof(T));
  if (e != cudaSuccess) return fail(QBC_E_NOMEM, "tree build scratch (%s, %lld items): %s", what, (long long)need,
                                    cudaGetErrorString(e));
  return QBC_OK;
}

int grid_for(int64_t n) {
  int64_t b = (n + 255) / 256;
  return (int)std::max<int64_t>(1, std::min<int64_t>(b, 65535));
}

}  // namespace

int64_t build_node_bound(int64_t n, int levels) {
  int64_t total = 1, w = 1;
  for (int l = 1; l <= levels; ++l) {
    w = w > ((int64_t)1 << 40) ? w : w * 8;
    total += std::min<int64_t>(n, w);
  }
  return total;
}

void build_release(BuildScratch* s) {
  void* ptrs[] = {s->key, s->cre, s->slot, s->slot_old, s->par, s->base, s->own, s->tab[0], s->tab[1], s->tab[2],
                  s->dense, s->blocksum, s->box};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  *s = BuildScratch();
}

int build_reserve(BuildScratch* s, int64_t n, int levels) {
  if (n > ((int64_t)1 << 29)) return fail(QBC_E_ARG, "tree build: %lld points exceed 2^29", (long long)n);
  const int64_t nodes = build_node_bound(n, levels);
  if (nodes > INT32_MAX) return fail(QBC_E_ARG, "tree build: up to %lld nodes exceed int32 indices", (long long)nodes);
  int rc = QBC_OK;
  if (s->points < n || !s->key) {
    const int64_t m = std::max<int64_t>(n, 1);
    if (!rc) rc = grow_buf(&s->key, 0, m, "keys");
    if (!rc) rc = grow_buf(&s->cre, 0, m, "creators");
    if (!rc) rc = grow_buf(&s->slot, 0, m, "slots");
    if (!rc) rc = grow_buf(&s->slot_old, 0, m, "slots");
    if (!rc) rc = grow_buf(&s->par, 0, m, "parents");
    if (!rc) rc = grow_buf(&s->base, 0, m, "node ids");
    if (!rc) rc = grow_buf(&s->own, 0, m, "levels");
    if (rc) return rc;
    s->points = m;
  }
  if (levels > kDense && (s->tab_points < n || !s->tab[0])) {
    const int64_t m = std::max<int64_t>(n, 1);
    for (int t = 0; t < 3 && !rc; ++t) rc = grow_buf(&s->tab[t], 0, 8 * m, "creator tables");
    if (rc) return rc;
    for (int t = 0; t < 3; ++t) {
      cudaError_t e = cudaMemset(s->tab[t], 0xFF, (size_t)8 * m * sizeof(uint32_t));
      if (e != cudaSuccess) return fail(QBC_E_CUDA, "tree build: clear creator tables: %s", cudaGetErrorString(e));
    }
    s->tab_points = m;
  }
  const int64_t nb = (n + kScanChunk - 1) / kScanChunk;
  if (s->blocks < nb || !s->blocksum) {
    rc = grow_buf(&s->blocksum, 0, std::max<int64_t>(nb, 1), "block sums");
    if (rc) return rc;
    s->blocks = std::max<int64_t>(nb, 1);
  }
  if (s->box_nodes < nodes || !s->box) {
    rc = grow_buf(&s->box, 0, 6 * nodes, "leaf boxes");
    if (rc) return rc;
    s->box_nodes = nodes;
  }
  if (!s->dense) rc = grow_buf(&s->dense, 0, kDenseEntries, "prefix tables");
  return rc;
}

int build_tree_async(const float* d_pts, const int32_t* d_octets, int64_t n, float basesize, int levels,
                     int64_t first_index, BuildScratch* s, int32_t* child, int32_t* model, uint32_t* rec,
                     int32_t* total, unsigned* err, cudaStream_t stream, int grid, int64_t* launches) {
  if (levels < 0 || levels > kMaxBuildLevels) return fail(QBC_E_ARG, "tree build: levels %d outside 0..21", levels);
  if (n < 0 || n > s->points) return fail(QBC_E_ARG, "tree build: %lld points beyond the reserved scratch", (long long)n);
  if (levels > kDense && s->dirty) {
    for (int t = 0; t < 3; ++t)
      if (cudaMemsetAsync(s->tab[t], 0xFF, (size_t)8 * s->tab_points * sizeof(uint32_t), stream) != cudaSuccess)
        return fail(QBC_E_CUDA, "tree build: reset creator tables");
  }
  s->dirty = true;
  int64_t L0 = *launches;
  const int g = std::max(1, std::min(grid, grid_for(n)));
  if (cudaMemsetAsync(s->dense, 0xFF, kDenseEntries * sizeof(uint32_t), stream) != cudaSuccess)
    return fail(QBC_E_CUDA, "tree build: reset prefix tables");
  if (n > 0)
    keys_kernel<<<g, 256, 0, stream>>>(d_pts, d_octets, n, basesize, levels, s->key, s->own, s->cre, s->slot,
                                       s->slot_old, s->par, err);
  ++*launches;
  auto table = [&](int l) -> uint32_t* {
    return l <= kDense ? s->dense + dense_offset(l) : s->tab[l % 3];
  };
  for (int l = 1; l <= levels + 1 && n > 0; ++l) {
    const bool pd = l <= levels && l <= kDense;
    const uint32_t* t_res = l >= 2 ? table(l - 1) : nullptr;
    uint32_t* t_clr = (l >= 3 && l - 2 > kDense) ? table(l - 2) : nullptr;
    uint32_t* t_prop = l <= levels ? table(l) : nullptr;
    const size_t smem = pd ? sizeof(uint32_t) << (3 * l) : 0;
    level_kernel<<<g, 256, smem, stream>>>(l, levels, n, s->key, s->own, s->cre, s->slot, s->slot_old, s->par, t_res,
                                           t_clr, t_prop, pd ? 1 : 0);
    ++*launches;
  }
  const int64_t nb = std::max<int64_t>(1, (n + kScanChunk - 1) / kScanChunk);
  scan_chunks_kernel<<<(unsigned)nb, kScanThreads, 0, stream>>>(s->own, s->key, n, levels, s->slot,
                                                                 levels > kDense ? table(levels) : nullptr,
                                                                 s->blocksum);
  scan_top_kernel<<<1, 1024, 0, stream>>>(s->blocksum, nb, total);
  scan_nodes_kernel<<<(unsigned)nb, kScanThreads, 0, stream>>>(s->own, s->key, n, levels, s->blocksum, s->base,
                                                                first_index, reinterpret_cast<int4*>(child), model,
                                                                s->box);
  *launches += 3;
  if (n > 0) {
    link_kernel<<<g, 256, 0, stream>>>(s->key, s->own, s->par, s->base, n, levels, child);
    ++*launches;
  }
  for (int l = levels - 1; l >= 0; --l) {
    box_kernel<<<l == 0 ? 1 : g, 256, 0, stream>>>(l, levels, s->key, s->own, s->base, n, child, s->box, rec);
    ++*launches;
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    *launches = L0;
    return fail(QBC_E_CUDA, "tree build: %s", cudaGetErrorString(e));
  }
  s->dirty = false;
  return QBC_OK;
}

namespace {

// ---- octree_remove_point (octree.c:182-218) for a batch of points ----
//
// Per point, the walk of octree_remove_point on the unedited tree: size
// halves from the basecube edge for levels + 1 steps; (int)(c / size) % 2 with
// C truncation and remainder; at level == levels the current node is the
// leaf, reported with its parent and the parent's octet. Points of different
// leaves do not meet (a removal only cuts a parent's link to its leaf), so
// the batch equals sequential calls once duplicates of a leaf are resolved:
// the first in input order removes it, the later ones find the link cut.
// key = leaf << 32 | point index, or ~0 when the point removes nothing.
__global__ void remove_walk_kernel(const int32_t* __restrict__ child, const int32_t* __restrict__ model,
                                   int64_t n_nodes, const float* __restrict__ pts, int64_t n, float basesize,
                                   int levels, uint64_t* __restrict__ keys, int32_t* __restrict__ parent,
                                   int8_t* __restrict__ poct) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float x = pts[3 * i], y = pts[3 * i + 1], z = pts[3 * i + 2];
    uint64_t key = ~0ull;
    float size = basesize;
    int32_t index = 0, lindex = 0;
    int loctet = 0;
    for (int level = 0; level < levels + 1; ++level) {
      size /= 2.0f;
      const float qx = x / size, qy = y / size, qz = z / size;
      // a float -> int conversion outside int range is undefined in C: skip
      if (!(fabsf(qx) < 2147483648.0f && fabsf(qy) < 2147483648.0f && fabsf(qz) < 2147483648.0f)) break;
      int octet = (int)qx % 2;
      const int yi = (int)qy % 2, zi = (int)qz % 2;
      if (yi == 0) octet += 2;
      if (zi == 0) octet += 4;
      if (level == levels) {
        key = ((uint64_t)(uint32_t)index << 32) | (uint64_t)i;
        parent[i] = lindex;
        poct[i] = (int8_t)loctet;
        break;
      }
      if (octet < 0) break;  // x <= -size: the reference would read oct[-1]
      lindex = index;
      loctet = octet;
      index = child[(int64_t)index * 8 + octet];
      if (index <= 0 || index >= n_nodes) break;  // empty link (or not a node of this tree)
    }
    keys[i] = key;
  }
}

// Sorted keys: the first point of each leaf cuts the parent's link and
// reports the leaf's model index and the parent node.
__global__ void remove_apply_kernel(const uint64_t* __restrict__ keys, int64_t n, int32_t* __restrict__ child,
                                    const int32_t* __restrict__ model, const int32_t* __restrict__ parent,
                                    const int8_t* __restrict__ poct, int32_t* __restrict__ modind,
                                    int32_t* __restrict__ octind, unsigned long long* __restrict__ removed) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t k = keys[j];
    if (k == ~0ull) continue;
    const uint32_t leaf = (uint32_t)(k >> 32);
    if (j > 0 && (uint32_t)(keys[j - 1] >> 32) == leaf) continue;
    const int64_t i = (int64_t)(k & 0xFFFFFFFFull);
    child[(int64_t)parent[i] * 8 + poct[i]] = 0;
    modind[i] = model[leaf];
    octind[i] = parent[i];
    atomicAdd(removed, 1ull);
  }
}

}  // namespace

int remove_points(int32_t* child, const int32_t* model, int64_t n_nodes, const float* d_pts, int64_t n,
                  float basesize, int levels, int32_t* d_modind, int32_t* d_octind, int64_t* removed,
                  cudaStream_t stream, int64_t* launches) {
  if (n <= 0) {
    if (removed) *removed = 0;
    return QBC_OK;
  }
  if (n >= (int64_t)0xFFFFFFFF) return fail(QBC_E_ARG, "tree remove: %lld points in one call", (long long)n);
  try {
    auto pol = thrust::cuda::par.on(stream);
    thrust::device_vector<uint64_t> keys(n);
    thrust::device_vector<int32_t> parent(n);
    thrust::device_vector<int8_t> poct(n);
    thrust::device_vector<unsigned long long> count(1, 0ull);
    cudaMemsetAsync(d_modind, 0xFF, (size_t)n * 4, stream);  // -1: nothing removed
    cudaMemsetAsync(d_octind, 0xFF, (size_t)n * 4, stream);
    remove_walk_kernel<<<grid_for(n), 256, 0, stream>>>(child, model, n_nodes, d_pts, n, basesize, levels,
                                                        thrust::raw_pointer_cast(keys.data()),
                                                        thrust::raw_pointer_cast(parent.data()),
                                                        thrust::raw_pointer_cast(poct.data()));
    thrust::sort(pol, keys.begin(), keys.end());
    remove_apply_kernel<<<grid_for(n), 256, 0, stream>>>(thrust::raw_pointer_cast(keys.data()), n, child, model,
                                                         thrust::raw_pointer_cast(parent.data()),
                                                         thrust::raw_pointer_cast(poct.data()), d_modind, d_octind,
                                                         thrust::raw_pointer_cast(count.data()));
    *launches += 3;  // walk, sort, apply
    unsigned long long h = 0;
    cudaError_t e = cudaMemcpyAsync(&h, thrust::raw_pointer_cast(count.data()), sizeof(h), cudaMemcpyDeviceToHost,
                                    stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) return fail(QBC_E_CUDA, "tree remove: %s", cudaGetErrorString(e));
    if (removed) *removed = (int64_t)h;
  } catch (const std::exception& ex) {
    return fail(QBC_E_NOMEM, "tree remove: %s", ex.what());
  }
  return QBC_OK;
}

}  // namespace qbc
