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

// Device-side input checks that cannot stop a kernel: the kernel records the
// fault in the context's error word and leaves the bad item out; the next
// call that synchronizes with the host (qbc_synchronize, qbc_tree_nodes,
// qbc_download_tree) reports it and clears the word.
enum DeviceError : unsigned {
  kErrBuildPoint = 1u,  // a point to build from was negative, too large or not finite
  kErrBuildOctet = 2u,  // an octet path entry was outside 0..7
  kErrSkinBone = 4u,    // a skinned point named a bone outside the bone set
  kErrMmaTimeout = 8u,  // a bounded wait for the tensor cores gave up (the kernel stopped early)
  kErrRecordOverflow = 16u,  // a split frame's record queue was full (pixels left unwritten)
};

// Scratch of the GPU tree build, owned by the context and reused by every
// build: it grows to the largest build seen, so repeated builds of up to that
// size allocate nothing.
struct BuildScratch {
  int64_t points = 0;        // per-point arrays hold this many points
  int64_t tab_points = 0;    // creator tables hold 8 entries per point for this many
  int64_t blocks = 0;        // prefix-sum block sums
  int64_t box_nodes = 0;     // exact leaf-cell boxes (6 int32 per node)
  uint64_t* key = nullptr;   // path key, 3 bits per level, root level most significant
  uint32_t* cre = nullptr;   // creator of the point's node at the last resolved level
  uint32_t* slot = nullptr;  // table slot of the last proposed level
  uint32_t* slot_old = nullptr;  // table slot of the level before it
  uint32_t* par = nullptr;   // creator of the parent of the point's first own node
  int32_t* base = nullptr;   // id of the point's first own node
  uint8_t* own = nullptr;    // first level whose node the point creates (levels + 1: none)
  uint32_t* tab[3] = {nullptr, nullptr, nullptr};  // creator tables of the deeper levels
  uint32_t* dense = nullptr;  // prefix tables of the top levels
  int32_t* blocksum = nullptr;
  int32_t* box = nullptr;
  bool dirty = false;        // a build stopped midway: tables must be reset
};

// Nodes a build of n points at `levels` can make: 1 + sum over levels l of
// min(n, 8^l).
int64_t build_node_bound(int64_t n, int levels);

// Grow the scratch for n points at `levels` (allocates only when it grows).
int build_reserve(BuildScratch* s, int64_t n, int levels);
void build_release(BuildScratch* s);

// Enqueue on `stream` the node array of inserting n points (d_pts, float3)
// or n octet paths (d_octets, `levels` per point) in order into an empty
// tree (octree_insert_point / octree_insert_path numbering, model indices
// first_index + i), with the leaf-box records (rec, 16 words per node) of
// every node that has children. child (8 int32 per node), model and rec
// must hold build_node_bound(n, levels) nodes; s must have been reserved for
// n points. No allocation and no host synchronisation: the node count is
// written to *total on the device, and a bad point or octet is left out and
// flagged in *err (DeviceError bits).
int build_tree_async(const float* d_pts, const int32_t* d_octets, int64_t n, float basesize, int levels,
                     int64_t first_index, BuildScratch* s, int32_t* child, int32_t* model, uint32_t* rec,
                     int32_t* total, unsigned* err, cudaStream_t stream, int grid, int64_t* launches);

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
