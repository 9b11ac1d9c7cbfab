// Internal interface of the path-tracing and shadow-ray kernels (pathtrace.cu).
#pragma once
#include "grt_internal.hpp"

namespace grt {

// Shading data of the scene: original vertices and triangles (the reference's scenedata
// arrays, rt/cuda/base.h:360-388) and one albedo per material id.
struct pt_scene {
    const float4 *vpos;
    const uint4 *tris;
    const float *albedo;
    uint32_t n_albedo;
};

struct pt_params_dev {
    uint32_t max_bounces;
    uint32_t rr_start;
    float rr_continue;
    float eps;
    uint64_t seed;
};

size_t compact_scratch_bytes(uint32_t n);
cudaError_t launch_compact_hits(const grt_hit *hits, uint32_t n, uint32_t *out_indices, uint32_t *count,
                                uint32_t *scratch, cudaStream_t st);
cudaError_t launch_shadow_rays(const pt_scene &ps, const float4 *rays, const grt_hit *hits, uint32_t n,
                               const float light[3], float eps, float4 *out_rays, uint32_t *count, uint32_t *scratch,
                               cudaStream_t st);

size_t wavefront_state_bytes();
cudaError_t launch_wavefront_init(const pt_scene &ps, const pt_params_dev &pp, const float4 *prim_rays,
                                  const grt_hit *prim_hits, const uint32_t *hit_list, const uint32_t *n_list,
                                  uint32_t n_paths, void *states, uint32_t *queue, float4 *rays,
                                  grt_path_result *results, uint32_t *n_queue, cudaStream_t st);
cudaError_t launch_wavefront_shade(const pt_scene &ps, const pt_params_dev &pp, uint32_t max_n, const uint32_t *n_in,
                                   const uint32_t *queue_in, const float4 *rays_in, const grt_hit *hits, void *states,
                                   uint32_t *n_out, uint32_t *queue_out, float4 *rays_out, grt_path_result *results,
                                   grt_hit *bounce_hits, cudaStream_t st);

cudaError_t launch_fused(const dev_scene &sc, const pt_scene &ps, const pt_params_dev &pp, const float4 *prim_rays,
                         const grt_hit *prim_hits, uint32_t n_primary, const uint32_t *hit_list,
                         const uint32_t *n_list, uint32_t n_paths,
                         grt_path_result *results, grt_hit *bounce_hits, const launch_params &lp, unsigned *err,
                         unsigned *counter, float4 *starts, cudaStream_t st);
int fused_blocks_per_sm(int block_threads, int stack_entries, int order, bool alpha, const spec_cfg &spec);
// Raises the dynamic shared-memory limit of the path-tracing kernels (once per device).
cudaError_t prepare_pt_kernels();

}  // namespace grt
