// Triangle BVH for the GB300 traversal kernels (replaces the DXR acceleration structure the
// reference builds through the driver, Source/Falcor/Scene/Scene.cpp:3092-3764 in
// ssteinberg/PLTFalcor).  Binary BVH, 64-byte nodes holding both children's boxes, triangles
// reordered into leaf order as three float4 each.
#pragma once

#include <cstdint>
#include <vector>

namespace plt {

// Both children's boxes in one 64-byte node (four 16-byte loads per visit).
struct alignas(16) BvhNode {
    float lmin[3], lmax[3];   // left child box
    float rmin[3], rmax[3];   // right child box
    int32_t left, right;      // >= 0: node index; < 0: leaf ~((first << 4) | (count - 1))
    int32_t pad0, pad1;
};
static_assert(sizeof(BvhNode) == 64, "BvhNode must stay 64 bytes");

constexpr int kLeafMaxTris = 8;
constexpr int32_t kNoChild = INT32_MIN;  // absent child (empty scene, single-leaf scene)

struct BvhBuildStats {
    uint32_t nodes = 0, leaves = 0, maxDepth = 0;
    double sahCost = 0.0;
};

// Builds the BVH over n triangles given as vertex triples (v[9*i .. 9*i+8]).  Outputs the node
// array and, for each leaf slot, the original triangle index (triOrder).
void buildBvh(const float* triVerts, uint32_t nTris, std::vector<BvhNode>& nodes, std::vector<uint32_t>& triOrder,
              BvhBuildStats* stats);

}  // namespace plt
