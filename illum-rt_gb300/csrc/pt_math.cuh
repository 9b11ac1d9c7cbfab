// Bounce sampling, shading and ray setup for the fused path-tracing loop and the shadow-ray
// step, usable on host and device.
//
// Every formula is evaluated with explicitly rounded IEEE operations (add, sub, mul, div,
// sqrt; nothing contracted into an FMA, no library transcendental), so the GPU and a CPU
// restatement compiled with -ffp-contract=off produce the same bits. That is what lets the
// hits of every bounce be compared exactly with the oracle.
//
// Sources restated:
//   * PCG32 stream per path: rng_pcg::set_sequence / uniform_uint / uniform_float
//     (libgi/random.h:59-96; O'Neill's PCG32);
//   * cosine-weighted hemisphere sample: cosine_sample_hemisphere + uniform_sample_disk
//     (libgi/sampling.h:13-17, 32-36), with cos/sin of 2*pi*u from sincos_turns below;
//   * alignment of a tangent-space sample with a normal: align (libgi/util.h:212-218);
//   * flipping the normal against the incoming direction: flip_normals_to_ray
//     (libgi/util.h:221-225);
//   * shadow ray length: ray::length_exclusive, t_max = distance - eps (libgi/rt.h:30).
#pragma once
#include <cfloat>
#include <cmath>
#include <cstdint>

#ifndef __CUDACC__
using std::signbit;
#endif

#ifdef __CUDACC__
#define GRT_HD __host__ __device__ __forceinline__
#else
#define GRT_HD inline
#endif

namespace grt {
namespace pm {

GRT_HD float mul(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}
GRT_HD float add(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}
GRT_HD float sub(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fsub_rn(a, b);
#else
    return a - b;
#endif
}
GRT_HD float div(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fdiv_rn(a, b);
#else
    return a / b;
#endif
}
GRT_HD float sqrt_rn(float a) {
#ifdef __CUDA_ARCH__
    return __fsqrt_rn(a);
#else
    return std::sqrt(a);
#endif
}
GRT_HD float u32_to_f(uint32_t x) {
#ifdef __CUDA_ARCH__
    return __uint2float_rn(x);
#else
    return (float)x;
#endif
}

struct f3 {
    float x, y, z;
};
GRT_HD f3 sub3(f3 a, f3 b) { return {sub(a.x, b.x), sub(a.y, b.y), sub(a.z, b.z)}; }
GRT_HD float dot3(f3 a, f3 b) { return add(add(mul(a.x, b.x), mul(a.y, b.y)), mul(a.z, b.z)); }
GRT_HD f3 cross3(f3 a, f3 b) {
    return {sub(mul(a.y, b.z), mul(a.z, b.y)), sub(mul(a.z, b.x), mul(a.x, b.z)), sub(mul(a.x, b.y), mul(a.y, b.x))};
}
GRT_HD f3 scale3(f3 a, float s) { return {mul(a.x, s), mul(a.y, s), mul(a.z, s)}; }
GRT_HD f3 normalize3(f3 a) { return scale3(a, div(1.0f, sqrt_rn(dot3(a, a)))); }

// PCG32 (rng_pcg, libgi/random.h:59-96).
struct pcg32 {
    uint64_t state, inc;
    GRT_HD uint32_t next() {
        const uint64_t old = state;
        state = old * 0x5851f42d4c957f2dULL + inc;
        const uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
        const uint32_t rot = (uint32_t)(old >> 59u);
        return (xs >> rot) | (xs << ((~rot + 1u) & 31u));
    }
    GRT_HD void set_sequence(uint64_t seq) {
        state = 0u;
        inc = (seq << 1u) | 1u;
        next();
        state += 0x853c49e6748fea9bULL;
        next();
    }
    // uniform_float: min(1 - 2^-24, float(u32) * 2^-32)
    GRT_HD float uniform() {
        const float f = mul(u32_to_f(next()), 0x1p-32f);
        return f < 0x1.fffffep-1f ? f : 0x1.fffffep-1f;
    }
};

// sin and cos of 2*pi*u for u in [0, 1): the quadrant comes from 4u (exact), the remaining
// angle x = frac(4u) * pi/2 in [0, pi/2) goes through the Taylor polynomials of sin (to x^13)
// and cos (to x^12) in Horner form. Coefficients are the float roundings of +-1/k!.
GRT_HD void sincos_turns(float u, float &s, float &c) {
    const float t4 = mul(u, 4.0f);
    const int q = (int)t4;
    const float x = mul(sub(t4, (float)q), 0x1.921fb6p+0f);
    const float x2 = mul(x, x);
    float ps = 0x1.612462p-33f;                 //  1/13!
    ps = add(mul(ps, x2), -0x1.ae6456p-26f);    // -1/11!
    ps = add(mul(ps, x2), 0x1.71de3ap-19f);     //  1/9!
    ps = add(mul(ps, x2), -0x1.a01a02p-13f);    // -1/7!
    ps = add(mul(ps, x2), 0x1.111112p-7f);      //  1/5!
    ps = add(mul(ps, x2), -0x1.555556p-3f);     // -1/3!
    ps = add(mul(ps, x2), 1.0f);
    const float sn = mul(ps, x);
    float pc = 0x1.1eed8ep-29f;                 //  1/12!
    pc = add(mul(pc, x2), -0x1.27e4fcp-22f);    // -1/10!
    pc = add(mul(pc, x2), 0x1.a01a02p-16f);     //  1/8!
    pc = add(mul(pc, x2), -0x1.6c16c2p-10f);    // -1/6!
    pc = add(mul(pc, x2), 0x1.555556p-5f);      //  1/4!
    pc = add(mul(pc, x2), -0.5f);               // -1/2!
    const float cs = add(mul(pc, x2), 1.0f);
    switch (q & 3) {
        case 0: s = sn; c = cs; break;
        case 1: s = cs; c = -sn; break;
        case 2: s = -sn; c = -cs; break;
        default: s = -cs; c = sn; break;
    }
}

// cosine_sample_hemisphere (libgi/sampling.h:13-17, 32-36)
GRT_HD f3 cosine_sample_hemisphere(float u0, float u1) {
    const float r = sqrt_rn(u0);
    float sn, cs;
    sincos_turns(u1, sn, cs);
    const float dx = mul(r, cs), dy = mul(r, sn);
    const float z = sub(sub(1.0f, mul(dx, dx)), mul(dy, dy));
    return {dx, dy, z > 0.f ? sqrt_rn(z) : 0.f};
}

// align (libgi/util.h:212-218): rotates a tangent-space sample to the frame of `axis`.
GRT_HD f3 align(f3 v, f3 axis) {
    const float s = signbit(axis.z) ? -1.0f : 1.0f;  // copysign(1, axis.z)
    const f3 w = {v.x, v.y, mul(v.z, s)};
    const f3 h = {axis.x, axis.y, add(axis.z, s)};
    const float k = div(dot3(w, h), add(1.0f, axis.z < 0.f ? -axis.z : axis.z));
    return {sub(mul(k, h.x), w.x), sub(mul(k, h.y), w.y), sub(mul(k, h.z), w.z)};
}

// Geometric normal of the triangle (a, b, c), normalised and flipped to face against `dir`
// (flip_normals_to_ray, libgi/util.h:221-225: flip when dot(dir, n) > 0).
GRT_HD f3 facing_normal(f3 a, f3 b, f3 c, f3 dir) {
    f3 n = normalize3(cross3(sub3(b, a), sub3(c, a)));
    if (dot3(dir, n) > 0.f) n = {-n.x, -n.y, -n.z};
    return n;
}

// Hit point o + t d, then moved by eps along the facing normal.
GRT_HD f3 offset_hit_point(f3 o, f3 d, float t, f3 n, float eps) {
    return {add(add(o.x, mul(t, d.x)), mul(eps, n.x)), add(add(o.y, mul(t, d.y)), mul(eps, n.y)),
            add(add(o.z, mul(t, d.z)), mul(eps, n.z))};
}

// Sky seen by an escaping path: 0.5 + 0.5 * d.y.
GRT_HD float sky(f3 d) { return add(0.5f, mul(0.5f, d.y)); }

// Running digest of a path's hits (FNV-1a over 32-bit words).
GRT_HD uint32_t digest_word(uint32_t h, uint32_t w) { return (h ^ w) * 16777619u; }
static const uint32_t kDigestSeed = 2166136261u;
static const uint32_t kMissWord = 0xFFFFFFFFu;

}  // namespace pm
}  // namespace grt
