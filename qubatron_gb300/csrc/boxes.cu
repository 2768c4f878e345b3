// Leaf bounding boxes of every node's children, for exact subtree pruning in
// the traversal.
//
// For every node the record holds, per child octet, the box of the leaf
// cells of that child's subtree, relative to the child's cube and rounded
// outward to 1/256 of its edge (8 bits per bound). A ray that misses a
// child's box (expanded by a margin far above the traversal's rounding) can
// reach no leaf of that subtree, so the walk may skip it: the first leaf hit,
// and so every pixel, stays the same, and only the count of nodes visited
// drops.
//
// Record of node i (8 x 8 bytes, one per child octet o): word x = xlo |
// xhi << 8 | ylo << 16 | yhi << 24, word y = zlo | zhi << 8. Bounds
// count cells of 1/256 of the child's edge from the child's x-min, y-max and
// z-max corner (y and z grow downward, as the octet bits do); a bound pair
// lo > hi marks a subtree without leaves.
//
// Levels: the build walks the tree breadth first from the root; the depth of
// the tree is the last level that holds nodes, and the boxes are valid for
// renders whose maxlevel is at least that depth. A node reached twice (not a
// tree: two parents or a cycle, found from each node's position in the
// breadth-first order), a child index outside the array (which the walk
// reports when it meets it) or a tree deeper than the shader's stack leaves
// the boxes unusable.

#include <cuda_runtime.h>
#include <thrust/device_vector.h>

#include <cstdint>
#include <vector>

#include "qbc_internal.h"
#include "qbcuda.h"

using qbc::fail;

namespace qbc {
namespace {

constexpr int kMaxDepth = QBC_MAX_LEVEL + 1;

int grid_of(int64_t n) {
  const int64_t b = (n + 255) / 256;
  return (int)(b < 1 ? 1 : (b > 4096 ? 4096 : b));
}

// Children of the nodes in [in_b, in_e) of `order` appended at the end of
// the order (the counter), each with its position in pos. One counter update
// per warp and pass: each lane takes its node's children, the warp reserves
// their total at once.
__global__ void expand_kernel(const int32_t* __restrict__ child, int64_t n, int32_t* __restrict__ order,
                              int32_t* __restrict__ pos, int64_t in_b, int64_t in_e,
                              unsigned long long* __restrict__ count) {
  const int lane = threadIdx.x & 31;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  // the loop's trip count is the same for the whole warp (ballots below)
  for (int64_t j0 = in_b + (blockIdx.x * (int64_t)blockDim.x + threadIdx.x - lane); j0 < in_e; j0 += stride) {
    const int64_t j = j0 + lane;
    int32_t c[8];
    uint32_t take = 0;
    bool outside = false;
    if (j < in_e) {
      const int32_t node = order[j];
      const int4* p = reinterpret_cast<const int4*>(child + (int64_t)node * 8);
      const int4 a = p[0], b = p[1];
      c[0] = a.x; c[1] = a.y; c[2] = a.z; c[3] = a.w;
      c[4] = b.x; c[5] = b.y; c[6] = b.z; c[7] = b.w;
#pragma unroll
      for (int o = 0; o < 8; ++o) {
        take |= (c[o] > 0 && c[o] < n) ? (1u << o) : 0u;
        // an index outside the array: the walk must meet it (it reports
        // it), so no boxes for this tree
        outside |= c[o] != 0 && !(c[o] > 0 && c[o] < n);
      }
    }
    const unsigned mine = (unsigned)__popc(take);
    unsigned incl = mine;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
      if (lane >= o) incl += v;
    }
    const unsigned total = __shfl_sync(0xFFFFFFFFu, incl, 31);
    const bool any_outside = __any_sync(0xFFFFFFFFu, outside);
    unsigned long long base = 0;
    if (lane == 31 && (total || any_outside))
      base = atomicAdd(count, (unsigned long long)total + (any_outside ? (unsigned long long)n + 1ull : 0ull));
    base = __shfl_sync(0xFFFFFFFFu, base, 31);
    unsigned long long k = base + (incl - mine);
#pragma unroll
    for (int o = 0; o < 8; ++o) {
      if ((take >> o) & 1u) {
        if ((int64_t)k < n) {  // past n: not a tree, detected on the host
          order[k] = c[o];
          pos[c[o]] = (int32_t)k;
        }
        ++k;
      }
    }
  }
}

// A node appended twice (two parents, or a cycle) keeps one of its positions
// in pos, so another position of it disagrees: then the array is not a tree.
__global__ void unique_kernel(const int32_t* __restrict__ order, const int32_t* __restrict__ pos, int64_t total,
                              unsigned int* __restrict__ dup) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < total; j += (int64_t)gridDim.x * blockDim.x)
    if (pos[order[j]] != (int32_t)j) *dup = 1u;
}

// Exact boxes in leaf cells relative to each node's cube, for the nodes of one
// level (children done). box: 6 ints per node (xlo xhi ylo yhi zlo zhi).
__global__ void box_level_kernel(const int32_t* __restrict__ child, int64_t n, const int32_t* __restrict__ order,
                                 int64_t b, int64_t e, int leaf_level, int32_t half_cells,
                                 int32_t* __restrict__ box) {
  for (int64_t j = b + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < e; j += (int64_t)gridDim.x * blockDim.x) {
    const int32_t node = order[j];
    int32_t r[6];
    if (leaf_level) {
      r[0] = r[1] = r[2] = r[3] = r[4] = r[5] = 0;
    } else {
      r[0] = r[2] = r[4] = 0x7fffffff;
      r[1] = r[3] = r[5] = -1;
      for (int o = 0; o < 8; ++o) {
        const int32_t c = child[(int64_t)node * 8 + o];
        if (!(c > 0 && c < n)) continue;
        const int32_t* cb = box + (int64_t)c * 6;
        if (cb[1] < cb[0]) continue;  // no leaves below
        const int32_t off[3] = {(o & 1) ? half_cells : 0, (o & 2) ? half_cells : 0, (o & 4) ? half_cells : 0};
        for (int k = 0; k < 3; ++k) {
          r[2 * k] = min(r[2 * k], cb[2 * k] + off[k]);
          r[2 * k + 1] = max(r[2 * k + 1], cb[2 * k + 1] + off[k]);
        }
      }
    }
    for (int k = 0; k < 6; ++k) box[(int64_t)node * 6 + k] = r[k];
  }
}

// Records of the nodes of one level: each child's box quantised outward to
// 1/256 of the child's edge (child_cells leaf cells).
__global__ void record_kernel(const int32_t* __restrict__ child, int64_t n, const int32_t* __restrict__ order,
                              int64_t b, int64_t e, int32_t child_cells, const int32_t* __restrict__ box,
                              uint32_t* __restrict__ rec) {
  for (int64_t j = b + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < e; j += (int64_t)gridDim.x * blockDim.x) {
    const int32_t node = order[j];
    uint32_t w[16];
    for (int k = 0; k < 16; ++k) w[k] = 0u;
    for (int o = 0; o < 8; ++o) {
      const int32_t c = child[(int64_t)node * 8 + o];
      uint32_t q[6] = {255u, 0u, 255u, 0u, 255u, 0u};  // empty
      if (c > 0 && c < n) {
        const int32_t* cb = box + (int64_t)c * 6;
        if (cb[0] <= cb[1]) {
          for (int k = 0; k < 3; ++k) {
            const int64_t lo = cb[2 * k], hi1 = (int64_t)cb[2 * k + 1] + 1;  // [lo, hi1) in leaf cells
            // in 1/256 of the edge: floor(lo * 256 / cells), ceil(hi1 * 256 / cells) - 1
            const int64_t ql = lo * 256 / child_cells;
            const int64_t qh = (hi1 * 256 + child_cells - 1) / child_cells - 1;
            q[2 * k] = (uint32_t)(ql < 0 ? 0 : (ql > 255 ? 255 : ql));
            q[2 * k + 1] = (uint32_t)(qh < 0 ? 0 : (qh > 255 ? 255 : qh));
          }
        }
      }
      w[2 * o] = q[0] | (q[1] << 8) | (q[2] << 16) | (q[3] << 24);
      w[2 * o + 1] = q[4] | (q[5] << 8);
    }
    uint4* dst = reinterpret_cast<uint4*>(rec + (int64_t)node * 16);
    for (int k = 0; k < 4; ++k) dst[k] = make_uint4(w[4 * k], w[4 * k + 1], w[4 * k + 2], w[4 * k + 3]);
  }
}

}  // namespace

int build_child_boxes(const int32_t* child, int64_t n, uint32_t* rec, cudaStream_t stream, int* depth,
                      int64_t* launches) {
  *depth = -1;
  if (n <= 0) return QBC_OK;
  try {
    thrust::device_vector<int32_t> order(n), pos(n);
    thrust::device_vector<unsigned long long> count(1);
    thrust::device_vector<unsigned int> dup(1);
    int32_t zero = 0;
    unsigned int no = 0u;
    cudaMemcpyAsync(thrust::raw_pointer_cast(order.data()), &zero, 4, cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(thrust::raw_pointer_cast(pos.data()), &zero, 4, cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(thrust::raw_pointer_cast(dup.data()), &no, 4, cudaMemcpyHostToDevice, stream);
    // breadth first: level L holds order[off[L], off[L+1])
    std::vector<int64_t> off = {0, 1};
    unsigned long long total = 1;
    cudaMemcpyAsync(thrust::raw_pointer_cast(count.data()), &total, 8, cudaMemcpyHostToDevice, stream);
    for (int L = 0; L <= kMaxDepth; ++L) {
      const int64_t b = off[L], e = off[L + 1];
      if (e == b) break;
      expand_kernel<<<grid_of(e - b), 256, 0, stream>>>(child, n, thrust::raw_pointer_cast(order.data()),
                                                         thrust::raw_pointer_cast(pos.data()), b, e,
                                                         thrust::raw_pointer_cast(count.data()));
      ++*launches;
      cudaError_t err = cudaMemcpyAsync(&total, thrust::raw_pointer_cast(count.data()), 8, cudaMemcpyDeviceToHost,
                                        stream);
      if (err == cudaSuccess) err = cudaStreamSynchronize(stream);
      if (err != cudaSuccess) return fail(QBC_E_CUDA, "box build: %s", cudaGetErrorString(err));
      if ((int64_t)total > n) return QBC_OK;  // a node reached twice: no boxes
      off.push_back((int64_t)total);
    }
    // every node once (the counter alone misses a node reached twice when
    // others are unreachable)
    {
      unique_kernel<<<grid_of(off.back()), 256, 0, stream>>>(thrust::raw_pointer_cast(order.data()),
                                                            thrust::raw_pointer_cast(pos.data()), off.back(),
                                                            thrust::raw_pointer_cast(dup.data()));
      ++*launches;
      unsigned int d = 0u;
      cudaError_t err = cudaMemcpyAsync(&d, thrust::raw_pointer_cast(dup.data()), 4, cudaMemcpyDeviceToHost, stream);
      if (err == cudaSuccess) err = cudaStreamSynchronize(stream);
      if (err != cudaSuccess) return fail(QBC_E_CUDA, "box build: %s", cudaGetErrorString(err));
      if (d) return QBC_OK;  // a node reached twice: no boxes
    }
    // the deepest level with nodes
    int D = 0;
    while (D + 2 < (int)off.size() && off[D + 2] > off[D + 1]) ++D;
    if (D > QBC_MAX_LEVEL) return QBC_OK;  // deeper than any render goes: no boxes
    thrust::device_vector<int32_t> box((size_t)n * 6);
    for (int L = D; L >= 0; --L) {
      const int64_t b = off[L], e = off[L + 1];
      box_level_kernel<<<grid_of(e - b), 256, 0, stream>>>(child, n, thrust::raw_pointer_cast(order.data()), b, e,
                                                            L == D ? 1 : 0, L == D ? 0 : (int32_t)(1 << (D - L - 1)),
                                                            thrust::raw_pointer_cast(box.data()));
      ++*launches;
    }
    for (int L = 0; L < D; ++L) {
      const int64_t b = off[L], e = off[L + 1];
      record_kernel<<<grid_of(e - b), 256, 0, stream>>>(child, n, thrust::raw_pointer_cast(order.data()), b, e,
                                                         (int32_t)(1 << (D - L - 1)),
                                                         thrust::raw_pointer_cast(box.data()), rec);
      ++*launches;
    }
    cudaError_t err = cudaStreamSynchronize(stream);
    if (err == cudaSuccess) err = cudaGetLastError();
    if (err != cudaSuccess) return fail(QBC_E_CUDA, "box build: %s", cudaGetErrorString(err));
    *depth = D;
  } catch (const std::exception& ex) {
    return fail(QBC_E_NOMEM, "box build: %s", ex.what());
  }
  return QBC_OK;
}

}  // namespace qbc
