// bvh_host.h — host-side BVH construction and the device node layout.
#pragma once
#include <cstdint>
#include <string>
#include <vector>
#include <vector_types.h>
#include "pyre_math.cuh"
#include "../../include/pyre_cuda.h"

namespace pyre {

struct Aabb {
    f3 lo, hi;
};

// Device BVH node: the two children of one binary node, 64 bytes, one cache
// line per visit. Children's boxes are stored in the parent so a visit tests
// both boxes with the node's four 16-byte loads.
//   a = (c0.lo.x, c0.hi.x, c0.lo.y, c0.hi.y)
//   b = (c1.lo.x, c1.hi.x, c1.lo.y, c1.hi.y)
//   c = (c0.lo.z, c0.hi.z, c1.lo.z, c1.hi.z)
//   d = (child0, child1, count0, count1)
// child with count > 0: leaf, child = first triangle (or instance) slot;
// count == 0 and child >= 0: interior node index; child < 0: empty slot.
struct alignas(16) GpuNode {
    float a[4];
    float b[4];
    float c[4];
    int32_t d[4];
};
static_assert(sizeof(GpuNode) == 64, "GpuNode is one 64-byte line");

// Builds the reference's binned-SAH binary BVH (bvh.rs:45-64,180-409) over
// arbitrary primitive bounds/centroids. Output uses the reference node layout
// (pyre_bvh2_node): DFS pre-order, left child = index + 1.
// `max_leaf` bounds the primitives of a leaf (MAX_PRIMS_PER_LEAF = 8,
// bvh.rs:14); with 1 every primitive gets its own leaf unless centroids
// coincide.
void build_bvh2(const std::vector<Aabb>& prim_bounds, const std::vector<f3>& prim_centroids,
                std::vector<pyre_bvh2_node>& nodes, std::vector<uint32_t>& prim_indices, uint32_t max_leaf = 8);

// Sets child `slot` (0 or 1) of a device node: its box, child and count.
void set_gpu_child(GpuNode& g, int slot, const Aabb& box, int32_t child, int32_t count);

// Per-triangle bounds and centroids as MeshInstance::build computes them
// (mesh.rs:77-87, triangle_bounds / triangle_centroid mesh.rs:32-40).
void triangle_bounds(const float* positions, const uint32_t* indices, uint32_t n_triangles,
                     std::vector<Aabb>& bounds, std::vector<f3>& centroids);

// Checks that a caller-supplied reference BVH is well formed (indices in
// range, every primitive referenced once). Returns false with a message.
bool validate_bvh2(const pyre_bvh2_node* nodes, uint32_t n_nodes, const uint32_t* prim, uint32_t n_prims,
                   std::string* why);

// Collapses a reference binary BVH into device nodes. `node_base` is the
// global index of the first emitted node, `slot_base` the global index of the
// first triangle/instance slot (leaf offsets are added to it). Returns the
// root's box. A root that is itself a leaf becomes one device node with an
// empty second child.
Aabb collapse_bvh2(const pyre_bvh2_node* nodes, uint32_t n_nodes, int32_t node_base, int32_t slot_base,
                   std::vector<GpuNode>& out);

// Wide device node (W = 4 or 8 children), 32 * W bytes, each field an array
// over the W child slots so a visit loads whole float4 rows:
//   lox[W] hix[W] loy[W] hiy[W] loz[W] hiz[W]  child boxes
//   child[W]  wide node index (count == 0), first triangle slot (count > 0),
//             -1 for an empty slot
//   count[W]  triangles of a leaf child, 0 otherwise
// Stored as a flat float array: field f of child k of node n is element
// (n * 8 + f) * W + k.
#ifndef PYRE_WIDE_FIELDS
#define PYRE_WIDE_FIELDS 8
#endif

// Collapses the binary device BVH below `root` (a node of `bin`) into wide
// nodes appended to `out` (8 * W floats each) in depth-first pre-order. Each
// wide node takes the two children of a binary node and then repeatedly
// opens the interior child with the largest surface area until it holds W
// children or only leaves. Boxes, leaves and triangle slots are the binary
// BVH's own, so a wide traversal tests the same triangles. Returns the wide
// index of the new root.
int32_t collapse_wide(const std::vector<GpuNode>& bin, int32_t root, int width, std::vector<float>& out);

// Instance BVHs of a scene built on the GPU (bvh_device.cu): device nodes in
// the GpuNode layout (each mesh's nodes from root[k], depth-first) and the
// triangle records of all meshes in slot order, both owned by the caller
// (cudaFree), plus each mesh's root box.
struct DeviceBlas {
    GpuNode* nodes = nullptr;
    uint64_t n_nodes = 0;
    float4* tris = nullptr;
    std::vector<int32_t> root;
    std::vector<Aabb> box;
};

}  // namespace pyre
