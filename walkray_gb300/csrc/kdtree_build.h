// kdtree_build.h — host construction of WalkRay's scene tree and its
// flattening into the device layout of wr_device.cuh.
#pragma once

#include <cstdint>
#include <vector>

#include "wr_device.cuh"

namespace wr {

// The reference tree in flat form.  Nodes are numbered in depth-first
// pre-order (left before right), root = 0.
struct HostTree {
    std::vector<int32_t> left, right;      // child node ids, -1 for a leaf
    std::vector<float> box;                // 6 per node: min xyz, max xyz
    std::vector<uint32_t> leaf_first;      // per node: first entry in leaf_tris (leaves)
    std::vector<uint32_t> leaf_count;      // per node: triangle count (leaves)
    std::vector<uint32_t> leaf_tris;       // triangle ids, reference leaf order
    uint32_t max_depth = 0;
    uint32_t num_leaves = 0;
    uint32_t num_nodes() const { return (uint32_t)left.size(); }
};

// Median-split build with the reference's rules (KDTree::build(BEST) ->
// splitBest, kdtree.cpp:141-258): per node, for x, y, z take the median of
// the node's distinct vertex coordinates, count triangles with any vertex
// <= median, keep the axis whose left fraction is closest to 1/2 (first axis
// on ties); stop at one triangle or a fraction of 0 or 1; partition keeping
// order.  `tris` holds global vertex indices.  Subtrees are built in
// parallel with OpenMP tasks; the result does not depend on the thread count.
HostTree build_reference_tree(const float* verts, uint32_t nv, const uint32_t* tris, uint32_t nt, int threads);

struct DeviceLayout {
    std::vector<NodePair> pairs;
    std::vector<TriRec> slots;
    std::vector<uint32_t> slot_of;  // global triangle id -> slot
    float root_lo[3], root_hi[3];
    uint32_t root_w0 = 0, root_w1 = LEAF_FLAG;
    float scene_mag = 0.f;
};

// Flattens the tree: one NodePair per internal node (its two children), in
// depth-first order; leaf triangles copied into TriRec slots in leaf order with
// each leaf's list reversed (see wr_device.cuh).
DeviceLayout layout_for_device(const HostTree& t, const float* verts, uint32_t nv, const uint32_t* tris,
                               const int32_t* tri_obj, const uint32_t* tri_local);

}  // namespace wr
