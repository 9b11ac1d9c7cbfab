// Direct lighting: the sampling and integration steps of the reference's CUDA "direct-wf"
// algorithm, usable on host and device.
//
// Restated from rt/cuda/bounce.cu and the libgi helpers it calls:
//   * light choice by power: distribution_1d (libgi/discrete_distributions.cpp:33-60) over
//     luma(trianglelight::power()) (rt/cuda/preprocessing.cpp:17-35, libgi/scene.cpp:518-527,
//     libgi/color.h:4-6), searched like k::lower_bound / k::sample_index (bounce.cu:148-171);
//   * a point on the light: uniform_sample_triangle (libgi/sampling.h:42-45) and k::sample_Li
//     (bounce.cu:178-208): shadow ray from the hit point, t_max = distance - eps, pdf =
//     t_max^2 / (cos_light * area), zero for a light facing away;
//   * k::sample_light (bounce.cu:210-250): an emissive hit adds its emission and casts no ray;
//   * direction sampling instead of light sampling: k::sample_uniform_dir (bounce.cu:33-73) with
//     uniform_sample_hemisphere (libgi/sampling.h:20-28), k::sample_cos_dir (bounce.cu:91-129)
//     with cosine_sample_hemisphere, both aligned to the normal facing the camera ray, and
//     k::integrate_dir (bounce.cu:341-375): the emission of whatever the ray hits;
//   * k::integrate_light (bounce.cu:380-410) with layered_gtr2 (bounce.cu:333-339): the
//     Fresnel-weighted mix of lambertian_reflection (bounce.cu:291-295) and gtr_coat_reflection
//     (bounce.cu:316-331, GGX ggx_d / ggx_g1 at bounce.cu:298-313, fresnel_dielectric at
//     libgi/util.h:91-106), times cos(theta), over the pdf; the frame buffer gets (radiance, 1).
// Differences, each for bit-reproducible CPU/GPU results and the synthetic scenes:
//   * every operation is an explicitly rounded add, sub, mul, div or sqrt in the reference's
//     order; normalize is v * (1 / sqrt(v . v)) (the reference's CUDA helper uses rsqrtf, whose
//     last bits are implementation-defined);
//   * normals are the triangles' geometric normals (the synthetic scenes carry no vertex
//     normals); the shading normal faces the camera ray (flip_normals_to_ray), a light's normal
//     follows its winding (lights are one-sided, as in sample_Li);
//   * the random numbers of a sample (three for a light sample, two for a direction) come from
//     a PCG32 stream per (pixel, sample) instead of the reference's per-frame uniform buffer;
//   * sin and cos of 2 pi u come from pm::sincos_turns instead of sinf / cosf.
#pragma once
#include "pt_math.cuh"

namespace grt {
namespace dl {

using pm::add;
using pm::div;
using pm::f3;
using pm::mul;
using pm::sqrt_rn;
using pm::sub;

constexpr float kPi = 3.14159265358979323846f;                       // pi (libgi/rt.h:15)
constexpr float kOneOverPi = (float)(1.0 / 3.14159265358979323846);  // one_over_pi (libgi/rt.h:16)
constexpr float kOneOver2Pi = (float)(1.0 / (2.0 * 3.14159265358979323846));  // one_over_2pi (libgi/rt.h:17)
constexpr float kEps = 1e-4f;  // ray::eps (libgi/rt.h:25)

// The sampling strategies (grt_direct_params::sampling).
enum : uint32_t { kSampleLight = 0, kSampleUniform = 1, kSampleCosine = 2 };

// One material of the table: albedo, emission, index of refraction, roughness.
struct material {
    float albedo[3], emissive[3], ior, roughness;
};

GRT_HD f3 add3(f3 a, f3 b) { return {add(a.x, b.x), add(a.y, b.y), add(a.z, b.z)}; }
GRT_HD f3 mul3(f3 a, f3 b) { return {mul(a.x, b.x), mul(a.y, b.y), mul(a.z, b.z)}; }
GRT_HD float len3(f3 a) { return sqrt_rn(pm::dot3(a, a)); }
GRT_HD float cdot(f3 a, f3 b) {
    const float x = pm::dot3(a, b);
    return x < 0.0f ? 0.0f : x;
}
GRT_HD float absdot(f3 a, f3 b) {
    const float x = pm::dot3(a, b);
    return x < 0.0f ? -x : x;
}
GRT_HD bool not_black(f3 c) { return c.x != 0.0f || c.y != 0.0f || c.z != 0.0f; }

// luma (libgi/color.h:4-6)
GRT_HD float luma(f3 c) { return add(add(mul(0.212671f, c.x), mul(0.715160f, c.y)), mul(0.072169f, c.z)); }

// fresnel_dielectric (libgi/util.h:91-106)
GRT_HD float fresnel_dielectric(float cos_wi, float ior_medium, float ior_material) {
    const float ei = cos_wi < 0.0f ? ior_material : ior_medium;
    const float et = cos_wi < 0.0f ? ior_medium : ior_material;
    float c = cos_wi < 0.0f ? -cos_wi : cos_wi;
    c = c < 0.0f ? 0.0f : (c > 1.0f ? 1.0f : c);
    const float sin_t = mul(div(ei, et), sqrt_rn(sub(1.0f, mul(c, c))));
    if (sin_t >= 1.0f) return 1.0f;
    const float rev = sub(1.0f, mul(sin_t, sin_t));
    const float cos_t = sqrt_rn(rev > 0.0f ? rev : 0.0f);
    const float rparl = div(sub(mul(et, c), mul(ei, cos_t)), add(mul(et, c), mul(ei, cos_t)));
    const float rperp = div(sub(mul(ei, c), mul(et, cos_t)), add(mul(ei, c), mul(et, cos_t)));
    return div(add(mul(rparl, rparl), mul(rperp, rperp)), 2.0f);
}

// tan2_theta (libgi/util.h:141-160)
GRT_HD float tan2_theta(float cos_t) {
    float s2 = sub(1.0f, mul(cos_t, cos_t));
    s2 = s2 < 0.0f ? 0.0f : s2;
    return div(s2, mul(cos_t, cos_t));
}

GRT_HD bool finite(float x) {
#ifdef __CUDA_ARCH__
    return isfinite(x);
#else
    return std::isfinite(x);
#endif
}

// ggx_d, ggx_g1 (rt/cuda/bounce.cu:298-313)
GRT_HD float ggx_d(float n_dot_h, float roughness) {
    if (n_dot_h <= 0.0f) return 0.0f;
    const float t2 = tan2_theta(n_dot_h);
    if (!finite(t2)) return 0.0f;
    const float a2 = mul(roughness, roughness);
    const float nh2 = mul(n_dot_h, n_dot_h);
    const float s = add(a2, t2);
    return div(a2, mul(mul(kPi, mul(nh2, nh2)), mul(s, s)));
}
GRT_HD float ggx_g1(float n_dot_v, float roughness) {
    if (n_dot_v <= 0.0f) return 0.0f;
    const float t2 = tan2_theta(n_dot_v);
    if (!finite(t2)) return 0.0f;
    return div(2.0f, add(1.0f, sqrt_rn(add(1.0f, mul(mul(roughness, roughness), t2)))));
}

// layered_gtr2 (rt/cuda/bounce.cu:333-339) with lambertian_reflection and gtr_coat_reflection
GRT_HD f3 layered_gtr2(f3 w_o, f3 w_i, f3 ns, const material &m) {
    const float F = fresnel_dielectric(absdot(ns, w_o), 1.0f, m.ior);
    const bool same = pm::dot3(w_i, ns) > 0.0f;
    const f3 diff = same ? f3{mul(kOneOverPi, m.albedo[0]), mul(kOneOverPi, m.albedo[1]), mul(kOneOverPi, m.albedo[2])}
                         : f3{0.0f, 0.0f, 0.0f};
    float spec = 0.0f;
    if (pm::dot3(ns, w_i) > 0.0f) {
        const float nv = cdot(ns, w_o), nl = cdot(ns, w_i);
        if (nv != 0.0f) {
            const f3 h = pm::normalize3(add3(w_o, w_i));
            const float nh = cdot(ns, h), hl = cdot(h, w_i);
            const float Fh = fresnel_dielectric(hl, 1.0f, m.ior);
            const float D = ggx_d(nh, m.roughness);
            const float G = mul(ggx_g1(nv, m.roughness), ggx_g1(nl, m.roughness));
            const float av = nv < 0.0f ? -nv : nv, al = nl < 0.0f ? -nl : nl;
            spec = div(mul(mul(Fh, D), G), mul(mul(4.0f, av), al));
        }
    }
    const float k = sub(1.0f, F);
    return {add(mul(k, diff.x), mul(F, spec)), add(mul(k, diff.y), mul(F, spec)), add(mul(k, diff.z), mul(F, spec))};
}

// k::lower_bound + k::sample_index (rt/cuda/bounce.cu:148-171) over n lights
GRT_HD uint32_t sample_light_index(uint32_t n, const float *f, const float *cdf, float integral, float xi, float &pdf) {
    int count = (int)n, first = 0, i = 0;
    while (count > 0) {
        i = first;
        const int step = count / 2;
        i += step;
        if (cdf[i] < xi) {
            first = ++i;
            count -= step + 1;
        } else {
            count = step;
        }
    }
    const int id = i > 0 ? i - 1 : i;
    pdf = div(f[id], integral);
    return (uint32_t)id;
}

// What one light sample of one hit produces (k::sample_light + k::sample_Li).
struct light_sample {
    f3 org, dir;
    float tmax;  // -FLT_MAX: no shadow ray
    f3 lcol;
    float pdf;
};

// from = the hit point o + t d; a, b, c the light triangle's vertices.
GRT_HD light_sample sample_li(f3 from, f3 a, f3 b, f3 c, f3 emissive, float x0, float x1) {
    light_sample s;
    const float su0 = sqrt_rn(x0);
    const float bb = sub(1.0f, su0), bg = mul(x1, su0);
    const float w = sub(sub(1.0f, bb), bg);
    const f3 target = {add(add(mul(w, a.x), mul(bb, b.x)), mul(bg, c.x)),
                       add(add(mul(w, a.y), mul(bb, b.y)), mul(bg, c.y)),
                       add(add(mul(w, a.z), mul(bb, b.z)), mul(bg, c.z))};
    const f3 e1 = pm::sub3(b, a), e2 = pm::sub3(c, a);
    const f3 n = pm::normalize3(pm::cross3(e1, e2));
    f3 wi = pm::sub3(target, from);
    const float area = mul(0.5f, len3(pm::cross3(e1, e2)));
    float tmax = len3(wi);
    wi = {div(wi.x, tmax), div(wi.y, tmax), div(wi.z, tmax)};
    tmax = sub(tmax, kEps);
    s.org = from;
    s.dir = wi;
    s.tmax = tmax;
    const float cos_l = pm::dot3(n, f3{-wi.x, -wi.y, -wi.z});
    if (cos_l <= 0.0f) {
        s.lcol = {0.0f, 0.0f, 0.0f};
        s.pdf = 0.0f;
    } else {
        s.lcol = emissive;
        s.pdf = div(mul(tmax, tmax), mul(cos_l, area));
    }
    return s;
}

// uniform_sample_hemisphere (libgi/sampling.h:20-26): z = u0, r = sqrt|1 - z^2|, phi = 2 pi u1.
GRT_HD f3 uniform_sample_hemisphere(float u0, float u1) {
    const float r0 = sub(1.0f, mul(u0, u0));
    const float r = sqrt_rn(r0 < 0.0f ? -r0 : r0);
    float sn, cs;
    pm::sincos_turns(u1, sn, cs);
    return {mul(r, cs), mul(r, sn), u0};
}

// The direction of a direction sample around the normal ns facing the camera ray and its pdf:
// k::sample_uniform_dir (bounce.cu:33-73: pdf one_over_2pi) and k::sample_cos_dir
// (bounce.cu:91-129: pdf one_over_pi * cdot(w_i, n)).
GRT_HD f3 sample_dir(uint32_t sampling, f3 ns, float x0, float x1, float &pdf) {
    if (sampling == kSampleCosine) {
        const f3 w = pm::align(pm::cosine_sample_hemisphere(x0, x1), ns);
        pdf = mul(kOneOverPi, cdot(w, ns));
        return w;
    }
    pdf = kOneOver2Pi;
    return pm::align(uniform_sample_hemisphere(x0, x1), ns);
}

// k::integrate_light (rt/cuda/bounce.cu:380-410) and k::integrate_dir (bounce.cu:341-375, with
// lcol the emission of the triangle the direction ray hit): brightness * f * cos(theta) / pdf
GRT_HD f3 integrate(f3 lcol, f3 w_o, f3 w_i, f3 ns, const material &m, float pdf) {
    const f3 f = layered_gtr2(w_o, w_i, ns, m);
    const float cos_t = cdot(w_i, ns);
    const f3 bf = mul3(lcol, f);
    return {div(mul(bf.x, cos_t), pdf), div(mul(bf.y, cos_t), pdf), div(mul(bf.z, cos_t), pdf)};
}

}  // namespace dl
}  // namespace grt
