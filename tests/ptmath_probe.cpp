// Test helper: the library's bounce-sampling and shading math (illum-rt_gb300/csrc/pt_math.cuh,
// dl_math.cuh) compiled for the host, exposed as extern "C" loops over arrays so that the tests
// can compare it with the reference's own code (oracle/_ref/libref_sampling.so) and with double
// precision. The headers are the ones the kernels include; on the host every operation is a
// plain IEEE float operation (compiled with -ffp-contract=off), on the device an explicitly
// rounded intrinsic, so both give the same bits (the GPU path-tracing tests check that through
// whole paths).
#include "dl_math.cuh"

using namespace grt;

extern "C" {

void ptm_pcg(uint64_t seq, uint32_t n, uint32_t *words, float *floats) {
    pm::pcg32 a, b;
    a.set_sequence(seq);
    b.set_sequence(seq);
    for (uint32_t i = 0; i < n; ++i) {
        words[i] = a.next();
        floats[i] = b.uniform();
    }
}

void ptm_sincos_turns(const float *u, uint32_t n, float *s, float *c) {
    for (uint32_t i = 0; i < n; ++i) pm::sincos_turns(u[i], s[i], c[i]);
}

void ptm_cosine_sample(const float *u0, const float *u1, uint32_t n, float *out3) {
    for (uint32_t i = 0; i < n; ++i) {
        const pm::f3 v = pm::cosine_sample_hemisphere(u0[i], u1[i]);
        out3[3 * i] = v.x, out3[3 * i + 1] = v.y, out3[3 * i + 2] = v.z;
    }
}

void ptm_uniform_hemisphere(const float *u0, const float *u1, uint32_t n, float *out3) {
    for (uint32_t i = 0; i < n; ++i) {
        const pm::f3 v = dl::uniform_sample_hemisphere(u0[i], u1[i]);
        out3[3 * i] = v.x, out3[3 * i + 1] = v.y, out3[3 * i + 2] = v.z;
    }
}

void ptm_align(const float *v3, const float *axis3, uint32_t n, float *out3) {
    for (uint32_t i = 0; i < n; ++i) {
        const pm::f3 r = pm::align({v3[3 * i], v3[3 * i + 1], v3[3 * i + 2]},
                                   {axis3[3 * i], axis3[3 * i + 1], axis3[3 * i + 2]});
        out3[3 * i] = r.x, out3[3 * i + 1] = r.y, out3[3 * i + 2] = r.z;
    }
}

void ptm_facing_normal(const float *a3, const float *b3, const float *c3, const float *dir3, uint32_t n,
                       float *out3) {
    for (uint32_t i = 0; i < n; ++i) {
        const pm::f3 r = pm::facing_normal({a3[3 * i], a3[3 * i + 1], a3[3 * i + 2]},
                                           {b3[3 * i], b3[3 * i + 1], b3[3 * i + 2]},
                                           {c3[3 * i], c3[3 * i + 1], c3[3 * i + 2]},
                                           {dir3[3 * i], dir3[3 * i + 1], dir3[3 * i + 2]});
        out3[3 * i] = r.x, out3[3 * i + 1] = r.y, out3[3 * i + 2] = r.z;
    }
}

void ptm_fresnel(const float *cos_wi, const float *ior_medium, const float *ior_material, uint32_t n, float *out) {
    for (uint32_t i = 0; i < n; ++i) out[i] = dl::fresnel_dielectric(cos_wi[i], ior_medium[i], ior_material[i]);
}

void ptm_tan2_theta(const float *cos_t, uint32_t n, float *out) {
    for (uint32_t i = 0; i < n; ++i) out[i] = dl::tan2_theta(cos_t[i]);
}

void ptm_ggx_d(const float *cos_t, const float *roughness, uint32_t n, float *out) {
    for (uint32_t i = 0; i < n; ++i) out[i] = dl::ggx_d(cos_t[i], roughness[i]);
}

void ptm_ggx_g1(const float *cos_t, const float *roughness, uint32_t n, float *out) {
    for (uint32_t i = 0; i < n; ++i) out[i] = dl::ggx_g1(cos_t[i], roughness[i]);
}

void ptm_luma(const float *rgb3, uint32_t n, float *out) {
    for (uint32_t i = 0; i < n; ++i) out[i] = dl::luma({rgb3[3 * i], rgb3[3 * i + 1], rgb3[3 * i + 2]});
}

}  // extern "C"
