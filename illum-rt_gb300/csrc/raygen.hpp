// Ray generation on the device: the incoherent test rays of the reference CUDA tracer
// (raygen.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace grt {

// n rays (two float4 each) between two balls placed in the scene's vertex extent; `bounds` is
// six uint32 of device scratch.
cudaError_t launch_incoherent_rays(const float4 *vpos, uint32_t nv, float r1, float r2, uint64_t seed, float4 *rays,
                                   uint32_t n, uint32_t *bounds, cudaStream_t st);

}  // namespace grt
