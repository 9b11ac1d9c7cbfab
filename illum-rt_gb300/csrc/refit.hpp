// Refit of a built tree to new vertex positions (refit.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace grt {

enum : unsigned { kRefitBadTree = 1u, kRefitNonFinite = 2u };

struct refit_args {
    const float4 *vpos;  // the new positions, already in the context's vertex array
    const uint4 *tris;
    uint32_t nv, nt;
    float4 *records;
    uint32_t n_records;
    float4 *nodes;         // binary nodes (bvh_builder.hpp layout)
    const int32_t *links;  // per node: (parent << 1) | side, -1 for the root or a node outside the tree
    uint32_t n_nodes;
    int32_t root;          // node index of the root (unused when n_nodes == 0)
    unsigned *arrive;      // n_nodes counters (scratch)
    unsigned *flags;       // kRefit* bits (device)
};

// Stream-ordered: records, then node boxes. The 4-wide nodes are rebuilt from the binary ones
// by the caller (gpu_build_wide).
cudaError_t launch_refit(const refit_args &a, cudaStream_t st);

}  // namespace grt
