// BVH construction on the GPU (top-down binned SAH, PLOC clustering or linear BVH, each with SAH
// leaf collapse), written in the device layout of bvh_builder.hpp: 64-byte binary nodes, 48-byte
// triangle records and 128-byte 4-wide nodes.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace grt {

// Per-scene results, written by the device into an int32[8] array.
enum gpu_build_info : int {
    GB_ROOT = 0,        // child reference of the binary root (a leaf reference if the tree is one leaf)
    GB_DEPTH = 1,       // edges from the root to the deepest leaf
    GB_ROOT4 = 2,       // child reference of the 4-wide root
    GB_BOUND4 = 3,      // most stack entries a 4-wide traversal can hold
    GB_ERR = 4,         // error bits (GB_ERR_*)
    GB_WIDE_NODES = 5,  // 4-wide nodes of the tree
    GB_INNER = 6,       // binary inner nodes reachable from the root
    GB_FINITE = 7,      // 1: every vertex coordinate of the scene is finite
};
enum : int { GB_ERR_INDEX = 1, GB_ERR_DEPTH = 2, GB_ERR_TREE = 4 };

// How the binary tree is formed: the radix tree of the Morton codes (linear BVH), agglomerative
// clustering in Morton order (PLOC), or top-down binned SAH splits (gpu_build_sah.cu).
enum : int { GB_METHOD_LBVH = 0, GB_METHOD_PLOC = 1, GB_METHOD_SAH = 2 };

// Most candidate planes per node of the SAH method.
constexpr int kMaxSahPlanes = 256;

// Scratch bytes for scenes of up to `max_tris` triangles built with `method`.
size_t gpu_build_scratch_bytes(uint32_t max_tris, int method);

// Phase 1 of one scene: binary nodes (max(nt - 1, 1) x 64 B), records (nt x 48 B), for every
// binary node its 4-wide node index (wide_index, nt ints, -1 for none) and, if `links` is not
// null, its refit link (nt ints: (parent << 1) | side for the inner nodes in the tree, -1
// elsewhere). `info` (int32[8], device) receives the fields above. Stream-ordered; the LBVH
// method reads nothing back, PLOC reads its cluster count back every 8 iterations (so that it
// stops launching once the tree is finished).
// `planes` (1 .. kMaxSahPlanes) is the SAH method's candidate count per node; the SAH method
// reads a node count back every 4 levels of its top part.
cudaError_t gpu_build_binary(const float4 *vpos, uint32_t nv, const uint4 *tris, uint32_t nt, int max_leaf,
                             void *scratch, size_t scratch_bytes, float4 *nodes, float4 *records,
                             int32_t *wide_index, int32_t *links, int32_t *info, int method, int planes,
                             cudaStream_t st);

// The SAH method's full binary tree over the n >= 2 primitives with boxes plo / phi (`bounds`:
// the ordered-encoded min corner then max corner of all of them): children, range and parent
// links in the radix tree's form, and the primitive order (*order, inside `scratch`). `flag`,
// `excl` (n ints) and the scan workspace are scratch of the caller.
size_t sah_scratch_bytes(uint32_t n);
cudaError_t sah_tree(void *scratch, uint32_t n, int planes, const float4 *plo, const float4 *phi,
                     const uint32_t *bounds, int2 *children, int2 *range, int32_t *parent_inner,
                     int32_t *parent_leaf, int32_t *flag, int32_t *excl, void *cub_tmp, size_t cub_bytes,
                     const uint32_t **order, int32_t *info, cudaStream_t st);

// Scene sets with the SAH method: the large-node levels of every scene's tree in one chain of
// launches over the set's primitives. Scene i holds the positions [first, first + n) of the
// set's arrays (plo / phi, the tree arrays, the order) and its inner nodes are numbered from
// first; `cbounds` holds 16 words per scene, the primitive pass's bounds. On return every array
// is in each scene's own numbering (positions, inner nodes and primitives from 0), so the
// slices at first are what sah_tree gives for the scene alone. `scenes` is on the device.
struct sah_set_scene {
    uint32_t first, n;
};
cudaError_t sah_tree_set(void *scratch, uint32_t n, const sah_set_scene *scenes, uint32_t count, int planes,
                         const float4 *plo, const float4 *phi, const uint32_t *cbounds, int2 *children,
                         int2 *range, int32_t *parent_inner, int32_t *parent_leaf, int32_t *flag, int32_t *excl,
                         void *cub_tmp, size_t cub_bytes, const uint32_t **order, int32_t *info, cudaStream_t st);

// A scene set's build with the SAH method in three phases (gpu_build.cu), over the arrays of
// one allocation: primitive boxes, the tree arrays and the SAH scratch for all primitives of
// the set, the primitive pass's bounds of every scene and the scene table.
constexpr uint32_t kSahSetMaxTris = 1u << 25;  // most primitives of one set (larger: several sets)
struct sah_set {
    float4 *lo, *hi;
    uint32_t *cbounds;  // 16 words per scene
    int2 *children, *range;
    int32_t *parent_inner, *parent_leaf, *flag, *excl;
    sah_set_scene *scenes;
    void *sah, *cub;
    size_t cub_bytes, total;
    uint32_t n, count;
};
sah_set sah_set_carve(void *base, uint32_t n_total, uint32_t count);  // base null: sizes only
// Phase 1, scene i of the set (stream-ordered): its info and bounds initialised, the boxes of
// its nt primitives written at positions first .. first + nt - 1 of the set's box arrays.
cudaError_t sah_set_prims(const sah_set &S, uint32_t i, uint32_t first, const float4 *vpos, uint32_t nv,
                          const uint4 *tris, uint32_t nt, int32_t *info, cudaStream_t st);
// Phase 2, every scene (after phase 1 of all of them; n_total >= 2): the scene table (host,
// scenes in position order) copied to the device, the parent links cleared, the trees built;
// *order receives the primitive order, `set_info` (int32[8], device) the GB_ERR bits of the
// trees of all scenes (OR-ed in).
cudaError_t sah_set_trees(const sah_set &S, const sah_set_scene *scenes_host, int planes, const uint32_t **order,
                          int32_t *set_info, cudaStream_t st);
// Phase 3, scene i (after phase 2): from its tree to the binary nodes, records and 4-wide
// indices, with `scratch` of gpu_build_scratch_bytes(nt, GB_METHOD_LBVH) bytes.
cudaError_t sah_set_finish(const sah_set &S, const uint32_t *order, uint32_t first, const float4 *vpos,
                           uint32_t nv, const uint4 *tris, uint32_t nt, int max_leaf, void *scratch,
                           size_t scratch_bytes, float4 *nodes, float4 *records, int32_t *wide_index, int32_t *info,
                           cudaStream_t st);

// A pinned host word for the builders' read-backs, one per host thread (a copy into pageable
// memory goes through a staging buffer that serialises the threads of a scene-set build).
int32_t *readback_word();

// Phase 2: the 4-wide nodes (info[GB_WIDE_NODES] x 128 B) from the binary nodes of phase 1.
cudaError_t gpu_build_wide(const float4 *nodes, const int32_t *wide_index, uint32_t nt, float4 *nodes4,
                           cudaStream_t st);

}  // namespace grt
