// Internal interface of the multi-scene traversal kernel (multi.cu).
#pragma once
#include "grt_internal.hpp"

namespace grt {

// One ray batch of a multi-scene launch, in device memory (32 bytes).
struct multi_batch {
    const float4 *rays;  // 2 float4 per ray
    grt_hit *hits;
    uint32_t offset;     // first global ray index of the batch (ascending over batches)
    uint32_t scene;      // index into the scene table
    uint32_t n;
    uint32_t pad;
};

cudaError_t launch_trace_multi(const dev_scene *scenes, const multi_batch *batches, uint32_t nbatch, uint32_t total,
                               bool any_hit, const launch_params &lp, unsigned *err, unsigned *counter,
                               cudaStream_t st);
cudaError_t prepare_multi_kernels();
int multi_blocks_per_sm(int block_threads, int stack_entries, int order, const spec_cfg &spec);

}  // namespace grt
