// Ray generation on the device: the camera rays of the primary-ray step and the incoherent test
// rays of the reference CUDA tracer (raygen.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace grt {

// n rays (two float4 each) between two balls placed in the scene's vertex extent; `bounds` is
// six uint32 of device scratch.
// w x h camera rays in cam_ray's arithmetic (cam: pos, dir, up, near_w, near_h as 11 floats);
// offsets: two floats per pixel or null (then PCG jitter from `seed` when `jitter`, else centres).
cudaError_t launch_camera_rays(const float cam[11], uint32_t w, uint32_t h, const float2 *offsets, bool jitter,
                               uint64_t seed, float4 *rays, cudaStream_t st);

cudaError_t launch_incoherent_rays(const float4 *vpos, uint32_t nv, float r1, float r2, uint64_t seed, float4 *rays,
                                   uint32_t n, uint32_t *bounds, cudaStream_t st);

}  // namespace grt
