// Direct lighting (the reference's "direct-wf" steps, light or direction sampling) in a
// wavefront form and a fused persistent form.
#pragma once
#include <cuda_runtime.h>

#include "dl_math.cuh"
#include "grt_internal.hpp"

namespace grt {

// Scene data of the direct-lighting kernels (device pointers).
struct dl_scene {
    const float4 *vpos;
    const uint4 *tris;
    const dl::material *mats;
    uint32_t n_mat;
    const uint4 *lights;  // emissive triangles: vertex indices, material id
    const float *lf;      // light power (luma)
    const float *lcdf;    // normalised cumulative power, n_lights + 1 entries
    uint32_t n_lights;
    float integral;       // sum of lf
};

// Wavefront step 1 for sample `s`: a sample of the strategy `sampling` (dl::kSample*) for every
// primary hit (emissive hits add their emission to fb), the rays to trace (t_max = -FLT_MAX
// where there is none), (light colour, pdf).
cudaError_t launch_dl_sample(const dl_scene &ds, const float4 *rays, const grt_hit *hits, uint32_t n, uint32_t s,
                             uint64_t seed, uint32_t sampling, float4 *shadow_rays, float4 *lsample, float4 *fb,
                             cudaStream_t st);
// Wavefront step 3: fb += (radiance, 1) from the traced rays' answers (any hit for light
// sampling, closest hit for the direction strategies).
cudaError_t launch_dl_integrate(const dl_scene &ds, const float4 *rays, const grt_hit *hits, const float4 *shadow_rays,
                                const grt_hit *shadow_hits, const float4 *lsample, uint32_t n, uint32_t sampling,
                                float4 *fb, cudaStream_t st);
// fb += (albedo, 1) of every hit (add_hitpoint_albedo), the wavefront form's shading launch.
cudaError_t launch_add_albedo(const dl_scene &ds, const grt_hit *hits, uint32_t n, float4 *fb, cudaStream_t st);
// The fused form: camera-ray traversal, `samples` samples with their ray traversals, and the
// integration, in one persistent launch, in any loop order. `albedo` != 0 adds
// add_hitpoint_albedo's (albedo, 1) of every camera ray before the samples.
cudaError_t launch_dl_fused(const dev_scene &sc, const dl_scene &ds, const float4 *rays, uint32_t n, uint32_t samples,
                            uint64_t seed, uint32_t sampling, uint32_t albedo, float4 *fb, int order,
                            int stack_entries, int block_threads, int num_sms, unsigned *err, unsigned *counter,
                            cudaStream_t st);
cudaError_t prepare_dl_kernels();

}  // namespace grt
