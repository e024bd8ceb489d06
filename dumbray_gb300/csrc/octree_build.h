// octree_build.h - host octree builder (flat, BFS-ordered output) for the GB300 ray caster.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace drb {

struct BuildOptions {
    int max_depth = 24;        // OCTREE_MAX_DEPTH (Octree.cuh:13)
    int split_threshold = 8;   // OCTREE_POLYCOUNT_TO_SPLIT_NODE (Octree.cuh:11)
    int threads = 0;           // 0 = all host cores
    // Padding of octant and leaf boxes: 0 = OCTREE_AABB_EPSILON (Octree.impl.cuh:3-5, 1.28e-3),
    // which casts and traversal counts of the reference require; > 0 = that absolute value;
    // < 0 = 2^-18 x the largest absolute coordinate.  The closest hit does not depend on it (up to
    // exact ties), so physical-mode scenes may use a value scaled to the coordinates.
    float box_eps = 0.0f;
    bool device = false;       // build on the GPU (build_octree_gpu), same tree
};

// Flattened octree.  The root is stored separately; the children of an inner node are 8
// consecutive nodes starting at node_child[i] (a multiple of 8), in octant order
// (bit 2 = upper x, bit 1 = upper y, bit 0 = upper z).  Leaves have node_child = -1 and own
// leaf_refs[node_leaf_first .. + node_leaf_count) (triangle indices in the reference's order).
struct FlatOctree {
    int64_t node_count = 0;
    std::vector<float> node_lo, node_hi;     // [node_count][3]
    std::vector<int32_t> node_child;         // [node_count]
    std::vector<int64_t> node_leaf_first;    // [node_count]
    std::vector<int32_t> node_leaf_count;    // [node_count]
    float root_lo[3] = {0, 0, 0}, root_hi[3] = {0, 0, 0};
    int32_t root_child = -1;                 // 0 when the root is split, -1 when it is a leaf
    int64_t root_leaf_first = 0;
    int32_t root_leaf_count = 0;
    std::vector<int32_t> leaf_refs;
    int depth = 0;
};

// xyz: float[n][3][3].  Returns false on invalid input.
bool build_octree(const float *xyz, int64_t n, const BuildOptions &opt, FlatOctree &out);

// The same build on the current CUDA device (octree_gpu.cu): per-reference clipping and per-node
// passes on the GPU, level bookkeeping on the host; bit-identical output.  err: reason on failure.
bool build_octree_gpu(const float *xyz, int64_t n, const BuildOptions &opt, FlatOctree &out, std::string &err);

}  // namespace drb
