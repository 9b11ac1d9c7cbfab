// Test-infrastructure harness around the reference's own sampling, camera and shading helpers.
//
// Compiled together with the UNMODIFIED reference source libgi/camera.cpp and the reference's
// header-only helpers (by oracle/build_ref.sh, into oracle/_ref/libref_sampling.so). It exposes,
// through extern "C" loops over arrays, the reference code that sits on either side of the
// traversal in the diffuse bounce and ray-setup steps, so that tests can pin the library's own
// versions of these steps against the reference itself:
//   * rng_pcg: set_sequence, uniform_uint, uniform_float (libgi/random.h:59-96);
//   * uniform_sample_disk, uniform_sample_hemisphere, cosine_sample_hemisphere
//     (libgi/sampling.h:13-36);
//   * align and flip_normals_to_ray (libgi/util.h:212-225);
//   * fresnel_dielectric and tan2_theta (libgi/util.h:91-106, 141-160), luma (libgi/color.h:4-6);
//   * camera::update_frustum and cam_ray (libgi/camera.h:7-24, libgi/camera.cpp:11-28).
// Only the tests load it; it never ships (the reference sources are not in this repository and
// the library is git-ignored).
#include "libgi/camera.h"
#include "libgi/color.h"
#include "libgi/random.h"
#include "libgi/rt.h"
#include "libgi/sampling.h"
#include "libgi/util.h"

#include <cstdint>

extern "C" {

// n words of uniform_uint and n values of uniform_float, each from its own generator started
// with set_sequence(seq).
void refs_pcg(uint64_t seq, uint32_t n, uint32_t *words, float *floats) {
    rng_pcg a(seq), b(seq);
    for (uint32_t i = 0; i < n; ++i) {
        words[i] = a.uniform_uint();
        floats[i] = b.uniform_float();
    }
}

// cosine_sample_hemisphere(vec2(u0[i], u1[i])) -> out3
void refs_cosine_sample(const float *u0, const float *u1, uint32_t n, float *out3) {
    for (uint32_t i = 0; i < n; ++i) {
        const vec3 v = cosine_sample_hemisphere(vec2(u0[i], u1[i]));
        out3[3 * i] = v.x, out3[3 * i + 1] = v.y, out3[3 * i + 2] = v.z;
    }
}

// uniform_sample_hemisphere(vec2(u0[i], u1[i])) -> out3
void refs_uniform_hemisphere(const float *u0, const float *u1, uint32_t n, float *out3) {
    for (uint32_t i = 0; i < n; ++i) {
        const vec3 v = uniform_sample_hemisphere(vec2(u0[i], u1[i]));
        out3[3 * i] = v.x, out3[3 * i + 1] = v.y, out3[3 * i + 2] = v.z;
    }
}

// align(v[i], axis[i]) -> out3
void refs_align(const float *v3, const float *axis3, uint32_t n, float *out3) {
    for (uint32_t i = 0; i < n; ++i) {
        const vec3 r = align(vec3(v3[3 * i], v3[3 * i + 1], v3[3 * i + 2]),
                             vec3(axis3[3 * i], axis3[3 * i + 1], axis3[3 * i + 2]));
        out3[3 * i] = r.x, out3[3 * i + 1] = r.y, out3[3 * i + 2] = r.z;
    }
}

// flip_normals_to_ray(normal[i], dir[i]) -> out3 (the normal, negated when it faces along dir)
void refs_flip(const float *normal3, const float *dir3, uint32_t n, float *out3) {
    for (uint32_t i = 0; i < n; ++i) {
        vec3 nrm(normal3[3 * i], normal3[3 * i + 1], normal3[3 * i + 2]);
        flip_normals_to_ray(nrm, vec3(dir3[3 * i], dir3[3 * i + 1], dir3[3 * i + 2]));
        out3[3 * i] = nrm.x, out3[3 * i + 1] = nrm.y, out3[3 * i + 2] = nrm.z;
    }
}

// fresnel_dielectric(cos_wi[i], ior_medium[i], ior_material[i]) -> out
void refs_fresnel(const float *cos_wi, const float *ior_medium, const float *ior_material, uint32_t n, float *out) {
    for (uint32_t i = 0; i < n; ++i) out[i] = fresnel_dielectric(cos_wi[i], ior_medium[i], ior_material[i]);
}

// tan2_theta(cos_t[i]) and luma(rgb[i]) -> out
void refs_tan2_theta(const float *cos_t, uint32_t n, float *out) {
    for (uint32_t i = 0; i < n; ++i) out[i] = tan2_theta(cos_t[i]);
}
void refs_luma(const float *rgb3, uint32_t n, float *out) {
    for (uint32_t i = 0; i < n; ++i) out[i] = luma(vec3(rgb3[3 * i], rgb3[3 * i + 1], rgb3[3 * i + 2]));
}

// The facing geometric normal of triangle (a, b, c) seen along dir: normalize(cross(b - a,
// c - a)) flipped by flip_normals_to_ray -> out3
void refs_facing_normal(const float *a3, const float *b3, const float *c3, const float *dir3, uint32_t n,
                        float *out3) {
    for (uint32_t i = 0; i < n; ++i) {
        const vec3 a(a3[3 * i], a3[3 * i + 1], a3[3 * i + 2]), b(b3[3 * i], b3[3 * i + 1], b3[3 * i + 2]);
        const vec3 c(c3[3 * i], c3[3 * i + 1], c3[3 * i + 2]);
        vec3 nrm = normalize(cross(b - a, c - a));
        flip_normals_to_ray(nrm, vec3(dir3[3 * i], dir3[3 * i + 1], dir3[3 * i + 2]));
        out3[3 * i] = nrm.x, out3[3 * i + 1] = nrm.y, out3[3 * i + 2] = nrm.z;
    }
}

// The reference camera (position, normalised view direction, up, vertical field of view in
// degrees, image size) and its cam_ray at every pixel centre, in the GPU ray layout
// (o.xyz, t_min, d.xyz, t_max) with ray index y * w + x; also returns near_w and near_h.
void refs_cam_rays(const float *pos3, const float *dir3, const float *up3, float fovy, int w, int h, float *rays8,
                   float *near_wh) {
    camera cam(vec3(dir3[0], dir3[1], dir3[2]), vec3(pos3[0], pos3[1], pos3[2]), vec3(up3[0], up3[1], up3[2]), fovy,
               w, h);
    near_wh[0] = cam.near_w;
    near_wh[1] = cam.near_h;
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) {
            const ray r = cam_ray(cam, x, y);
            float *o = rays8 + 8 * ((size_t)y * w + x);
            o[0] = r.o.x, o[1] = r.o.y, o[2] = r.o.z, o[3] = r.t_min;
            o[4] = r.d.x, o[5] = r.d.y, o[6] = r.d.z, o[7] = r.t_max;
        }
}

// cam_ray at every pixel of a camera given as the struct's fields (near_w and near_h set
// directly rather than from a field of view), with sub-pixel offsets: offsets2 (two floats per
// pixel) when given; otherwise, with jitter != 0, (uniform_float() - 0.5, uniform_float() - 0.5)
// from rng_pcg(seed + pixel index); otherwise the pixel centres.
void refs_cam_rays_offsets(const float *pos3, const float *dir3, const float *up3, float near_w, float near_h, int w,
                           int h, const float *offsets2, int jitter, uint64_t seed, float *rays8) {
    camera cam(vec3(dir3[0], dir3[1], dir3[2]), vec3(pos3[0], pos3[1], pos3[2]), vec3(up3[0], up3[1], up3[2]), 60.0f,
               w, h);
    cam.near_w = near_w;
    cam.near_h = near_h;
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) {
            const size_t i = (size_t)y * w + x;
            vec2 off(0.0f, 0.0f);
            if (offsets2) {
                off = vec2(offsets2[2 * i], offsets2[2 * i + 1]);
            } else if (jitter) {
                rng_pcg rng(seed + i);
                const float ox = rng.uniform_float() - 0.5f;
                const float oy = rng.uniform_float() - 0.5f;
                off = vec2(ox, oy);
            }
            const ray r = cam_ray(cam, x, y, off);
            float *o = rays8 + 8 * i;
            o[0] = r.o.x, o[1] = r.o.y, o[2] = r.o.z, o[3] = r.t_min;
            o[4] = r.d.x, o[5] = r.d.y, o[6] = r.d.z, o[7] = r.t_max;
        }
}

}  // extern "C"
