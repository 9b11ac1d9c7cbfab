// Host-side BVH construction and flattening for the GB300 traversal kernels.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace grt {

// One node of the reference's binary BVH (bbvh_node, rt/cpu/bvh.h:42-52): two child boxes and
// two links; a leaf stores link_l = -first, link_r = -count (positions in `index`).
struct ref_node {
    float lmin[3], lmax[3], rmin[3], rmax[3];
    int32_t link_l, link_r;
    bool inner() const { return link_r >= 0; }
};

struct ref_tree {
    uint32_t root = 0;
    std::vector<ref_node> nodes;  // preorder, as the reference numbers them
    std::vector<uint32_t> index;  // leaf slot -> triangle id (ESC fragments repeat ids)
};

struct build_opts {
    int split = 2;  // 0 object median, 1 spatial median, 2 SAH
    int max_tris = 4;
    int planes = 16;
    bool esc = true;
    int threads = 0;  // 0 = hardware concurrency
};

// Builds the reference's BVH (rt/cpu/bvh-ctor.h:96-503) over float4 vertices and uint4
// triangles. Returns false with a message for inputs the reference cannot build.
bool build_reference_bvh(const float *vpos4, uint32_t nv, const uint32_t *tris4, uint32_t nt,
                         const build_opts &opts, ref_tree &out, std::string &err);

// Device layout produced from a reference tree.
//
// Node (64 bytes): two 32-byte child records, left then right, each
//   (min.x, min.y, max.x, max.y, min.z, max.z, child reference as int bits, 0)
// so that the slab test's x/y bounds pair with the ray's (o.x, o.y) and the z bounds with
// (o.z, o.z) as packed f32x2 operands (traverse.cuh).
// A child reference c >= 0 is an inner node index; c < 0 is a leaf with ~c = (first << 4) |
// (count - 1), `first` indexing the triangle records, so leaves never need a fetch of their own.
// Triangle record (48 bytes, three float4), in leaf order:
//   [0] v0.xyz, w = original triangle id (int bits)
//   [1] v0 - v1 (the a, b, c of the reference's Cramer test, libgi/intersect.h:27-29), w = material id
//   [2] v0 - v2 (d, e, f, libgi/intersect.h:32-34)
// Subtracting on the host in float gives the same bits as the reference's per-test subtraction.
struct flat_bvh {
    std::vector<float> nodes;    // 16 floats per inner node
    std::vector<float> records;  // 12 floats per record
    std::vector<int32_t> parent;    // per inner node: (parent << 1) | side, -1 for the root (refit)
    std::vector<int32_t> inner_id;  // per reference node: its inner node index, -1 for a leaf
    int32_t root = 0;            // child reference of the root (a leaf reference if the tree is one leaf)
    uint32_t depth = 0;          // edges from the root to the deepest leaf
    uint32_t inner = 0;
    bool empty = false;          // no triangles: every ray misses
};

static const uint32_t kMaxLeafTris = 16;
static const uint32_t kMaxRecords = 1u << 27;

bool flatten_bvh(const ref_tree &tree, const float *vpos4, const uint32_t *tris4, flat_bvh &out, std::string &err);

// 4-wide device layout: the reference tree collapsed two levels at a time. A wide node holds
// the children of a binary node's inner children (the grandchildren) and its leaf children,
// 2 to 4 of them, with their boxes as the reference stores them. 128 bytes: four 32-byte child
// records in the binary node's format, (lo.x, lo.y, hi.x, hi.y, lo.z, hi.z, reference, 0); a
// reference >= 0 is a wide node, < 0 a leaf (same encoding and the same triangle records as the
// binary layout), kEmptyChild an unused slot (its box all +inf).
// Children appear in the reference's left-to-right order; wide nodes are in preorder.
static const int32_t kEmptyChild = 0x7fffffff;
struct flat_bvh4 {
    std::vector<float> nodes;  // 32 floats per wide node
    std::vector<int32_t> wide_index;  // per binary inner node and one more: the wide node it heads, -1 for none
    int32_t root = 0;          // wide node 0, or a leaf reference if the tree is one leaf
    uint32_t count = 0;
    uint32_t stack_bound = 0;  // most stack entries a traversal can hold
};

bool flatten_bvh4(const ref_tree &tree, const flat_bvh &flat, flat_bvh4 &out, std::string &err);

}  // namespace grt
