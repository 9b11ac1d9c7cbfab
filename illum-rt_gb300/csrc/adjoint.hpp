// Internal interface of the adjoint kernel (adjoint.cu).
#pragma once
#include "grt_internal.hpp"

namespace grt {

// grad_tbg: 3 floats per ray (dL/dt, dL/dbeta, dL/dgamma). vpos: vstride floats per vertex.
// grad_v (optional): 3 floats per vertex, accumulated. grad_rays (optional): 2 float4 per ray.
cudaError_t launch_adjoint(const float4 *rays, const grt_hit *hits, const float *grad_tbg, uint32_t n,
                           const float4 *vpos, uint32_t vstride, const uint4 *tris, float *grad_v, float4 *grad_rays,
                           cudaStream_t st);

}  // namespace grt
