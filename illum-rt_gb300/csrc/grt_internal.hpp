// Internal interfaces between the C-ABI (api.cpp) and the kernels (*.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/grt.h"

namespace grt {

// Everything a traversal kernel needs about one scene; passed by value as a kernel argument.
// Texture data of the alpha-aware tracers (device memory, one allocation).
struct alpha_data {
    const uint4 *tris;       // the scene's triangles: vertex indices, material id
    const float2 *tc;        // texture coordinate per vertex
    const int32_t *mat_tex;  // texture per material, -1 for none
    const uint4 *tex;        // per texture: width, height, first texel, 0
    const float *texels;     // alpha values, texture after texture, row by row
    uint32_t n_mat;
};

struct dev_scene {
    const float4 *nodes;    // 4 float4 per inner node (layout in bvh_builder.hpp)
    const float4 *records;  // 3 float4 per triangle record
    const float4 *nodes4;   // 8 float4 per 4-wide node (flat_bvh4)
    int32_t root;           // child reference of the root
    int32_t root4;          // child reference of the 4-wide root
    int32_t empty;          // 1: no triangles, every ray misses
    int32_t finite;         // 1: every vertex coordinate is finite (enables the min/max slab test)
    const alpha_data *alpha;  // alpha-aware tracing, or nullptr
};

// Bits a kernel ORs into the context's error word.
enum : unsigned { ERR_STACK_OVERFLOW = 1u, ERR_STEP_LIMIT = 2u, ERR_ABORTED = 4u };

// The context's status block in device memory: [0] error bits, [1] work counter of the
// persistent kernels, [32] abort request (alone in its 128-byte line, away from the counter's
// atomics). Kernels receive a pointer to word 0 (`err`). To stop work, the host writes the
// abort request and a huge value into the counter, both with copy-engine writes on a stream of
// their own so that they land while kernels run: a running persistent kernel then finds its
// counter exhausted at its next fetch and ends, with no extra work in its loop, and a
// persistent kernel that starts later reads the request once per warp on entry and does
// nothing. One-thread-per-ray kernels are not stopped: each is bounded by its ray count.
enum : int { kStatusErr = 0, kStatusCounter = 1, kStatusAbort = 32, kStatusWords = 64 };
static const unsigned kAbortCounter = 0xC0000000u;  // far beyond any ray count, far below 2^32

#ifdef __CUDACC__
// Warp-uniform entry check: true (and ERR_ABORTED recorded) when the host has asked the
// context's kernels to stop. All 32 lanes must call it before any lane leaves.
__device__ __forceinline__ bool stop_requested_at_entry(unsigned *err) {
    unsigned stop = 0;
    if ((threadIdx.x & 31u) == 0) {
        stop = *((const volatile unsigned *)(err + kStatusAbort)) != 0u ? 1u : 0u;
        if (stop) atomicOr(err, ERR_ABORTED);
    }
    return __shfl_sync(0xffffffffu, stop, 0) != 0u;
}
#endif

// Largest traversal stack (entries per thread, in shared memory) a launch may ask for; a
// launch allocates exactly the entries it asks for (the tree's depth unless tuned deeper).
static const int kStackLarge = 64;

// The speculative loop order's warp-level parameters (traverse.cuh): how many leaves a lane may
// postpone before the warp's leaf phase (1 to 3), with how many lanes still searching for their
// first leaf the warp stops visiting nodes, and how many node visits each lane makes between two
// warp votes. Launch arguments; the defaults per kernel family are the ones measured best on
// GB300, and the persistent families (fused path tracer, persistent traces, scene sets) take
// the tuned values of grt_tuning when set.
struct spec_cfg {
    int pend, exit, visits;
};
// The launch functions refuse (cudaErrorInvalidValue) parameters outside these ranges.
inline bool spec_ok(const spec_cfg &c) {
    return c.pend >= 1 && c.pend <= 3 && c.exit >= 0 && c.exit <= 32 && c.visits >= 1 && c.visits <= 16;
}
// Kernel instances of the speculative order compiled for common (visits per vote, postponed
// leaves) pairs, whose node loop the compiler unrolls and whose unused postponement slots it
// drops (2 % off the fused path step on GB300 against the run-time form); instance 0 takes the
// values at run time. fast_path_of picks the instance of a configuration.
constexpr int kFastPaths = 5;
constexpr int kFastVisits[kFastPaths] = {0, 5, 3, 3, 5};
constexpr int kFastPend[kFastPaths] = {0, 2, 2, 3, 3};
inline int fast_path_of(const spec_cfg &c) {
    for (int f = 1; f < kFastPaths; ++f)
        if (c.visits == kFastVisits[f] && c.pend == kFastPend[f]) return f;
    return 0;
}

constexpr spec_cfg kSpecPaths = {2, 8, 5};       // fused path tracer
constexpr spec_cfg kSpecDirect = {3, 2, 3};      // fused direct lighting
constexpr spec_cfg kSpecTrace = {3, 1, 3};       // one-thread-per-ray batch traces
constexpr spec_cfg kSpecPersistent = {2, 8, 3};  // persistent batch traces, scene sets

// Upper bound on traversal steps (inner nodes + leaves) of one ray. A DFS over a tree visits
// each node at most once per ray, so a correct BVH never reaches it; it bounds the work of a
// kernel given a corrupted tree.
static const uint32_t kStepLimit = 1u << 26;

// Loop orders of the traversal kernels (traverse.cuh): one node or leaf per iteration; inner
// nodes until a leaf and then that leaf; speculative while-while (postponed leaves, results
// equal to the reference's except near-ties); the speculative order over 4-wide nodes (the
// same near-tie guarantee).
enum loop_order : int { IF_IF = 0, WHILE_WHILE = 1, SPECULATIVE = 2, WIDE_SPECULATIVE = 3 };
static const int32_t kEmptyWideChild = 0x7fffffff;  // unused slot of a 4-wide node

struct launch_params {
    int block_threads;
    int grid_blocks;        // persistent kernels: total resident blocks
    int refill_threshold;
    int refill_period;
    int stack_entries;             // traversal stack entries per thread (the launch's shared memory)
    spec_cfg spec;                 // speculative order: the family default or the tuned values
    int order;                     // loop_order
    unsigned long long *counters;  // one-thread-per-ray kernel: rays, inner nodes, triangle tests (or null)
};

// `n_dev` (optional): the ray count is read on the device from *n_dev (at most n); the grid
// still covers n rays.
cudaError_t launch_trace_plain(const dev_scene &sc, const float4 *rays, grt_hit *hits, uint32_t n, bool any_hit,
                               const launch_params &lp, unsigned *err, cudaStream_t stream,
                               const uint32_t *n_dev = nullptr);

cudaError_t launch_trace_persistent(const dev_scene &sc, const float4 *rays, grt_hit *hits, uint32_t n, bool any_hit,
                                    const launch_params &lp, unsigned *err, unsigned *counter, cudaStream_t stream);

// Raises the dynamic shared-memory limit of every traversal kernel variant (once per device,
// before any launch, so that launches need no attribute calls and can be captured).
cudaError_t prepare_trace_kernels();

// Occupancy of the persistent kernel for a block size and stack size (blocks per SM), of the
// instance that a launch with speculative parameters `spec` runs.
int persistent_blocks_per_sm(int block_threads, int stack_entries, bool any_hit, int order, bool alpha,
                             const spec_cfg &spec);

}  // namespace grt
