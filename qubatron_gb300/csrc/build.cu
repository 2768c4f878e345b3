// GPU node-array builder: the same node array as inserting points one by one
// with octree_insert_point (src/qubatron/octree.c:95-147) or octet paths with
// octree_insert_path (octree.c:149-180) into an empty tree, numbering
// included, without the sequential walk.
//
// Sequential insertion appends a node the first time a path prefix appears:
// point i walks down the nodes earlier points made and appends the rest of
// its path. So the node of a prefix is created by the smallest point index
// having that prefix, and point i creates exactly the levels [c_i, levels)
// where c_i is the first level whose prefix it owns. Node ids follow from one
// prefix sum of (levels - c_i) over points in index order:
//   id(i, L) = 1 + sum_{j < i} (levels - c_j) + (L - c_i).
// Steps: path keys -> sort by key -> per level, the runs of equal prefixes
// (reduce_by_key, min index) -> c_i by atomic min -> prefix sum -> ids ->
// each node links itself into its parent (binary search of the parent's
// prefix one level up).

#include <cuda_runtime.h>
#include <thrust/binary_search.h>
#include <thrust/device_vector.h>
#include <thrust/execution_policy.h>
#include <thrust/functional.h>
#include <thrust/iterator/transform_iterator.h>
#include <thrust/reduce.h>
#include <thrust/scan.h>
#include <thrust/sort.h>

#include <cstdint>
#include <vector>

#include "qbc_internal.h"
#include "qbcuda.h"

using qbc::fail;

namespace qbc {
namespace {

constexpr int kMaxBuildLevels = 21;  // 3 bits per level in a 64-bit key

// Octets of octree.c:100-109 (and skeleton_vsh.c:195-204 for in-cube
// points): size halves from the basecube edge, (int)(x / size) % 2 picks the
// x bit, y and z below the midline set bits 1 and 2.
__global__ void point_keys_kernel(const float* __restrict__ pts, int64_t n, float basesize, int levels,
                                  uint64_t* __restrict__ keys, uint32_t* __restrict__ idx, int* __restrict__ bad) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float x = pts[3 * i], y = pts[3 * i + 1], z = pts[3 * i + 2];
    uint64_t k = 0;
    if (!(x >= 0.0f && x < 1.0e30f && y >= 0.0f && y < 1.0e30f && z >= 0.0f && z < 1.0e30f)) {
      atomicExch(bad, 1);
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
    keys[i] = k;
    idx[i] = (uint32_t)i;
  }
}

__global__ void path_keys_kernel(const int32_t* __restrict__ octets, int64_t n, int levels,
                                 uint64_t* __restrict__ keys, uint32_t* __restrict__ idx, int* __restrict__ bad) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    uint64_t k = 0;
    for (int level = 0; level < levels; ++level) {
      int o = octets[i * levels + level];
      if (o < 0 || o > 7) {
        atomicExch(bad, 1);
        o = 0;
      }
      k = (k << 3) | (uint64_t)o;
    }
    keys[i] = k;
    idx[i] = (uint32_t)i;
  }
}

struct ShiftKey {
  int shift;
  __host__ __device__ uint64_t operator()(uint64_t k) const { return k >> shift; }
};

// Level at which each creator point starts creating nodes.
__global__ void first_level_kernel(const uint32_t* __restrict__ first, int64_t u, int level, int* __restrict__ c) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < u; k += (int64_t)gridDim.x * blockDim.x)
    atomicMin(&c[first[k]], level);
}

__global__ void count_kernel(const int* __restrict__ c, int64_t n, int levels, int64_t* __restrict__ cnt) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    cnt[i] = levels - c[i];
}

__global__ void ids_kernel(const uint32_t* __restrict__ first, int64_t u, int level, const int* __restrict__ c,
                           const int64_t* __restrict__ base, int32_t* __restrict__ ids) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < u; k += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t f = first[k];
    ids[k] = (int32_t)(1 + base[f] + (level - c[f]));
  }
}

// Link each node of a level into its parent and set its model index.
__global__ void link_kernel(const uint64_t* __restrict__ prefix, const uint32_t* __restrict__ first,
                            const int32_t* __restrict__ ids, int64_t u, const uint64_t* __restrict__ pprefix,
                            const int32_t* __restrict__ pids, int64_t pu, int64_t first_index,
                            int32_t* __restrict__ child, int32_t* __restrict__ model) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < u; k += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t p = prefix[k];
    int32_t parent = 0;
    if (pprefix) {
      const uint64_t want = p >> 3;
      int64_t lo = 0, hi = pu - 1;  // the parent prefix is present: binary search
      while (lo < hi) {
        int64_t mid = (lo + hi) >> 1;
        if (pprefix[mid] < want)
          lo = mid + 1;
        else
          hi = mid;
      }
      parent = pids[lo];
    }
    const int32_t id = ids[k];
    child[(int64_t)parent * 8 + (int)(p & 7)] = id;
    model[id] = (int32_t)(first[k] + first_index);
  }
}

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

int grid_for(int64_t n) {
  int64_t b = (n + 255) / 256;
  return (int)std::max<int64_t>(1, std::min<int64_t>(b, 65535));
}

}  // namespace

// Builds into caller-given device buffers that build_grow() sized.
int build_nodes(const float* d_pts, const int32_t* d_octets, int64_t n, float basesize, int levels,
                int64_t first_index, cudaStream_t stream, BuildTarget* tgt) {
  if (levels < 0 || levels > kMaxBuildLevels) return fail(QBC_E_ARG, "tree build: levels %d outside 0..21", levels);
  if (n < 0 || n > 0xFFFFFFFFll) return fail(QBC_E_ARG, "tree build: %lld points outside 0..2^32-1", (long long)n);
  auto pol = thrust::cuda::par.on(stream);
  int64_t total = 1;
  std::vector<thrust::device_vector<uint64_t>> prefix(levels);
  std::vector<thrust::device_vector<uint32_t>> first(levels);
  std::vector<thrust::device_vector<int32_t>> ids(levels);
  std::vector<int64_t> ucount(levels, 0);
  try {
    if (n > 0 && levels > 0) {
      thrust::device_vector<uint64_t> keys(n);
      thrust::device_vector<uint32_t> idx(n);
      thrust::device_vector<int> bad(1, 0);
      if (d_pts)
        point_keys_kernel<<<grid_for(n), 256, 0, stream>>>(d_pts, n, basesize, levels,
                                                            thrust::raw_pointer_cast(keys.data()),
                                                            thrust::raw_pointer_cast(idx.data()),
                                                            thrust::raw_pointer_cast(bad.data()));
      else
        path_keys_kernel<<<grid_for(n), 256, 0, stream>>>(d_octets, n, levels, thrust::raw_pointer_cast(keys.data()),
                                                           thrust::raw_pointer_cast(idx.data()),
                                                           thrust::raw_pointer_cast(bad.data()));
      tgt->launches += 1;
      int hbad = 0;
      cudaMemcpyAsync(&hbad, thrust::raw_pointer_cast(bad.data()), sizeof(int), cudaMemcpyDeviceToHost, stream);
      cudaStreamSynchronize(stream);
      if (hbad)
        return fail(QBC_E_ARG, d_pts ? "tree build: a point is negative, too large or not finite"
                                     : "tree build: an octet is outside 0..7");
      thrust::sort_by_key(pol, keys.begin(), keys.end(), idx.begin());
      {
        // one n-sized scratch pair reused by every level; each level keeps
        // only its unique prefixes
        thrust::device_vector<uint64_t> sp(n);
        thrust::device_vector<uint32_t> sf(n);
        for (int L = 0; L < levels; ++L) {
          auto kb = thrust::make_transform_iterator(keys.begin(), ShiftKey{3 * (levels - 1 - L)});
          auto end = thrust::reduce_by_key(pol, kb, kb + n, idx.begin(), sp.begin(), sf.begin(),
                                           thrust::equal_to<uint64_t>(), thrust::minimum<uint32_t>());
          ucount[L] = end.first - sp.begin();
          prefix[L].assign(sp.begin(), sp.begin() + ucount[L]);
          first[L].assign(sf.begin(), sf.begin() + ucount[L]);
        }
      }
      keys.clear();
      keys.shrink_to_fit();
      idx.clear();
      idx.shrink_to_fit();
      thrust::device_vector<int> c(n, levels);
      for (int L = 0; L < levels; ++L)
        first_level_kernel<<<grid_for(ucount[L]), 256, 0, stream>>>(thrust::raw_pointer_cast(first[L].data()),
                                                                    ucount[L], L, thrust::raw_pointer_cast(c.data()));
      thrust::device_vector<int64_t> cnt(n), base(n);
      count_kernel<<<grid_for(n), 256, 0, stream>>>(thrust::raw_pointer_cast(c.data()), n, levels,
                                                    thrust::raw_pointer_cast(cnt.data()));
      thrust::exclusive_scan(pol, cnt.begin(), cnt.end(), base.begin(), (int64_t)0);
      tgt->launches += levels + 1;
      for (int L = 0; L < levels; ++L) total += ucount[L];
      if (total > INT32_MAX) return fail(QBC_E_ARG, "tree build: %lld nodes exceed int32 indices", (long long)total);
      for (int L = 0; L < levels; ++L) {
        ids[L].resize(ucount[L]);
        ids_kernel<<<grid_for(ucount[L]), 256, 0, stream>>>(thrust::raw_pointer_cast(first[L].data()), ucount[L], L,
                                                            thrust::raw_pointer_cast(c.data()),
                                                            thrust::raw_pointer_cast(base.data()),
                                                            thrust::raw_pointer_cast(ids[L].data()));
      }
      tgt->launches += levels;
    }
    int rc = tgt->grow(tgt, total);
    if (rc) return rc;
    cudaMemsetAsync(tgt->child, 0, (size_t)total * 32, stream);
    cudaMemsetAsync(tgt->model, 0, (size_t)total * 4, stream);
    for (int L = 0; L < levels && n > 0; ++L) {
      link_kernel<<<grid_for(ucount[L]), 256, 0, stream>>>(
          thrust::raw_pointer_cast(prefix[L].data()), thrust::raw_pointer_cast(first[L].data()),
          thrust::raw_pointer_cast(ids[L].data()), ucount[L],
          L > 0 ? thrust::raw_pointer_cast(prefix[L - 1].data()) : nullptr,
          L > 0 ? thrust::raw_pointer_cast(ids[L - 1].data()) : nullptr, L > 0 ? ucount[L - 1] : 0, first_index,
          tgt->child, tgt->model);
    }
    tgt->launches += levels;
    cudaError_t e = cudaStreamSynchronize(stream);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) return fail(QBC_E_CUDA, "tree build: %s", cudaGetErrorString(e));
  } catch (const std::exception& ex) {
    return fail(QBC_E_NOMEM, "tree build: %s", ex.what());
  }
  tgt->n_nodes = total;
  return QBC_OK;
}

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
