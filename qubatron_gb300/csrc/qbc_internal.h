// Internal helpers shared by the translation units of libqbcuda.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "qbcuda.h"

namespace qbc {

// Record a message for qbc_last_error() and return `code`.
int fail(int code, const char* fmt, ...);
void clear_error();

// True when every cube coordinate of the view's traversal is exactly
// representable, so a child shift can be undone exactly on the way up.
bool cube_shift_exact(const qbc_view& v);

// Destination of a GPU tree build: grow() must make child (8 int32 per node)
// and model (1 int32 per node) hold `nodes` nodes on the device.
struct BuildTarget {
  int32_t* child;
  int32_t* model;
  int64_t n_nodes;
  int64_t launches;
  void* user;
  int (*grow)(BuildTarget* self, int64_t nodes);
};

// Build the node array of inserting n points (d_pts, float3) or n octet
// paths (d_octets, `levels` per point) in order into an empty tree. Inputs
// are device pointers; exactly one of d_pts / d_octets is non-null.
int build_nodes(const float* d_pts, const int32_t* d_octets, int64_t n, float basesize, int levels,
                int64_t first_index, cudaStream_t stream, BuildTarget* tgt);

// octree_remove_point (octree.c:182-218) of n points in order, on a device
// tree (child: 8 int32 per node, model: 1 per node): cuts the links in place,
// reports modind / octind per point (-1 where nothing was removed) into
// device arrays and the number removed.
int remove_points(int32_t* child, const int32_t* model, int64_t n_nodes, const float* d_pts, int64_t n,
                  float basesize, int levels, int32_t* d_modind, int32_t* d_octind, int64_t* removed,
                  cudaStream_t stream, int64_t* launches);

// Leaf-box records of every node's children (boxes.cu) for the tree `child`
// (8 int32 per node, n nodes) into rec (16 words per node); depth gets the
// tree's depth, or -1 when the array is not a tree the renders can use.
int build_child_boxes(const int32_t* child, int64_t n, uint32_t* rec, cudaStream_t stream, int* depth,
                      int64_t* launches);

}  // namespace qbc
