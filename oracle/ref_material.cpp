// Test-infrastructure harness around the reference's microfacet helpers.
//
// The reference's CPU shading code (libgi/material.cpp, included here unmodified as part of this
// translation unit, because its ggx_d and ggx_g1 are file-local inline functions) holds the same
// GGX normal-distribution and Smith masking terms as its CUDA direct-lighting kernels
// (rt/cuda/bounce.cu:298-313). Built into oracle/_ref/libref_sampling.so by oracle/build_ref.sh;
// only the tests load it.
#include "libgi/material.cpp"

// The harness builds no scene; the reference's destructor lives in libgi/scene.cpp, which needs
// assimp and is not compiled here.
scene::~scene() {}

extern "C" {

// ggx_d(n_dot_h[i], roughness[i]) and ggx_g1(n_dot_v[i], roughness[i]) -> out (libgi/material.cpp:237-260)
void refs_ggx_d(const float *cos_t, const float *roughness, uint32_t n, float *out) {
    for (uint32_t i = 0; i < n; ++i) out[i] = ggx_d(cos_t[i], roughness[i]);
}
void refs_ggx_g1(const float *cos_t, const float *roughness, uint32_t n, float *out) {
    for (uint32_t i = 0; i < n; ++i) out[i] = ggx_g1(cos_t[i], roughness[i]);
}

}  // extern "C"
