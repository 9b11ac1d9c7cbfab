// ORACLE — test infrastructure only. Never linked into, loaded by or called from the product.
//
// The oracle's own generators of the benchmark workload: the 256-sphere scene and pinhole
// camera rays. The CPU baseline and the reference arm of the benchmark build their inputs
// here, so that timing the reference's CPU tracer loads nothing but the oracle. The definitions
// are the workload's (seeded PCG32 stream, UV spheres with coincident pole vertices, pixel-centre
// rays of the reference's cam_ray construction, libgi/camera.cpp:11-28); a CPU test checks that
// the arrays equal the library's workload generators bit for bit.
//
// Everything is computed in double with IEEE add, subtract, multiply, divide and sqrt only
// (all correctly rounded on x86-64 and aarch64), then rounded once to float; compiled with
// -ffp-contract=off. No libm transcendental is called: the sphere angles are multiples of
// pi/16, whose cosines follow exactly from nested square roots (half-angle formulas), and the
// camera's tangent comes from Horner-evaluated Maclaurin polynomials of sine and cosine.
#include <cfloat>
#include <cmath>
#include <cstdint>

namespace orc_scenes {

// PCG32 (O'Neill 2014): state advance by the 64-bit LCG, output by xorshift and a random
// rotation; a stream is selected by its sequence number (the increment).
struct pcg {
    uint64_t s, inc;
    explicit pcg(uint64_t seq) : s(0), inc((seq << 1u) | 1u) {
        step();
        s += 0x853c49e6748fea9bULL;
        step();
    }
    uint32_t step() {
        const uint64_t x = s;
        s = x * 6364136223846793005ULL + inc;
        const uint32_t v = (uint32_t)(((x >> 18u) ^ x) >> 27u);
        const uint32_t r = (uint32_t)(x >> 59u);
        return (v >> r) | (v << ((32u - r) & 31u));
    }
    // 53 random bits as a double in [0, 1): 27 high bits, then 26 low bits
    double unit() {
        const uint64_t a = step() >> 5, b = step() >> 6;
        return (double)(a * (1ull << 26) + b) / 9007199254740992.0;
    }
};

// cos(k pi / 16) for k = 0..8 from the half-angle identity cos(x/2) = sqrt((1 + cos x) / 2)
// written as sqrt(2 + 2 cos x) / 2 with exact square roots of sums of square roots.
struct sixteenths {
    double c[33], s[33];
    sixteenths() {
        const double r2 = std::sqrt(2.0);
        const double a = std::sqrt(2.0 + r2), b = std::sqrt(2.0 - r2);
        double q[9];
        q[0] = 1.0;
        q[1] = std::sqrt(2.0 + a) / 2.0;
        q[2] = a / 2.0;
        q[3] = std::sqrt(2.0 + b) / 2.0;
        q[4] = r2 / 2.0;
        q[5] = std::sqrt(2.0 - b) / 2.0;
        q[6] = b / 2.0;
        q[7] = std::sqrt(2.0 - a) / 2.0;
        q[8] = 0.0;
        // cos over a full turn (k = 0..32) by the quarter-turn symmetries, sin(x) = cos(x - pi/2)
        for (int k = 0; k <= 32; ++k) {
            const int m = k % 32;
            double v;
            if (m <= 8) v = q[m];
            else if (m <= 16) v = -q[16 - m];
            else if (m <= 24) v = -q[m - 16];
            else v = q[32 - m];
            c[k] = v;
        }
        for (int k = 0; k <= 32; ++k) s[k] = c[(k + 24) % 32];
    }
};

struct d3 {
    double x, y, z;
};
inline d3 operator-(d3 a, d3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline d3 operator+(d3 a, d3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline d3 operator*(d3 a, double k) { return {a.x * k, a.y * k, a.z * k}; }
inline double dot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline d3 cross(d3 a, d3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline d3 unit(d3 a) { return a * (1.0 / std::sqrt(dot(a, a))); }

// tan x for |x| <= pi/4 as the quotient of the Maclaurin polynomials of sin and cos (terms up
// to x^23 and x^22), each evaluated in Horner form.
double tan_small(double x) {
    const double x2 = x * x;
    double sn = 1.0, cs = 1.0;
    for (int k = 11; k >= 1; --k) {
        sn = 1.0 - sn * x2 / double((2 * k) * (2 * k + 1));
        cs = 1.0 - cs * x2 / double((2 * k - 1) * (2 * k));
    }
    return (sn * x) / cs;
}

const double kPi = 3.141592653589793238462643383279502884;

}  // namespace orc_scenes

using namespace orc_scenes;

extern "C" {

// `count` UV spheres of `slices` x `stacks` quads (slices and stacks dividing 32), two triangles
// per quad, the pole rows of `slices` coincident vertices; centres U[-cext, cext]^3 and radii
// U[rmin, rmax] drawn in that order per sphere from one stream. Returns 0 on success, -1 for
// unsupported slice or stack counts.
int orc_scene_spheres(uint64_t seed, uint32_t count, uint32_t slices, uint32_t stacks, float cext, float rmin,
                      float rmax, float *vpos4, uint32_t *tris4) {
    if (slices == 0 || stacks == 0 || 32 % slices != 0 || 32 % (2 * stacks) != 0) return -1;
    static const sixteenths tab;
    pcg rng(seed);
    const uint32_t per_v = (stacks + 1) * slices, per_t = 2 * slices * stacks;
    for (uint32_t s = 0; s < count; ++s) {
        const double cx = (2 * rng.unit() - 1) * cext;
        const double cy = (2 * rng.unit() - 1) * cext;
        const double cz = (2 * rng.unit() - 1) * cext;
        const double r = rmin + (rmax - rmin) * rng.unit();
        for (uint32_t i = 0; i <= stacks; ++i) {
            const uint32_t ki = i * (16 / stacks);  // polar angle i pi / stacks in sixteenths of pi
            const bool pole = i == 0 || i == stacks;
            const double st = pole ? 0.0 : tab.s[ki];
            const double ct = i == 0 ? 1.0 : (i == stacks ? -1.0 : tab.c[ki]);
            for (uint32_t j = 0; j < slices; ++j) {
                const uint32_t kj = j * (32 / slices);  // azimuth 2 j pi / slices
                float *v = vpos4 + 4 * (size_t)(s * per_v + i * slices + j);
                v[0] = (float)(cx + r * st * tab.c[kj]);
                v[1] = (float)(cy + r * ct);
                v[2] = (float)(cz + r * st * tab.s[kj]);
                v[3] = 1.0f;
            }
        }
        for (uint32_t i = 0; i < stacks; ++i)
            for (uint32_t j = 0; j < slices; ++j) {
                const uint32_t j1 = (j + 1) % slices;
                const uint32_t a = s * per_v + i * slices + j, b = s * per_v + i * slices + j1;
                const uint32_t c = a + slices, d = b + slices;
                uint32_t *t = tris4 + 4 * (size_t)(s * per_t + 2 * (i * slices + j));
                t[0] = a, t[1] = c, t[2] = d, t[3] = s;
                t[4] = a, t[5] = d, t[6] = b, t[7] = s;
            }
    }
    return 0;
}

// Pinhole rays through the pixel centres of a w x h image, ray (x, y) at index y w + x: the
// reference's cam_ray construction (libgi/camera.cpp:11-28) with the near plane at distance 1,
// half height tan(fovy / 2) and half width scaled by the aspect ratio. Returns -1 for a field
// of view outside (0, 180) degrees.
int orc_camera_rays(const float *pos3, const float *look3, const float *up3, float fovy_deg, uint32_t w, uint32_t h,
                    float tmin, float *rays8) {
    if (!(fovy_deg > 0.f && fovy_deg < 180.f)) return -1;
    const d3 pos = {pos3[0], pos3[1], pos3[2]};
    const d3 dir = unit(d3{look3[0], look3[1], look3[2]} - pos);
    const d3 U = unit(cross(dir, d3{up3[0], up3[1], up3[2]}));
    const d3 V = unit(cross(U, dir));
    const double half = kPi * double(fovy_deg) * 0.5 / 180.0;
    // tan of angles above pi/4 through tan x = 1 / tan(pi/2 - x)
    const double th = half <= kPi / 4 ? tan_small(half) : 1.0 / tan_small(kPi / 2 - half);
    const double tw = th * double(w) / double(h);
    for (uint32_t y = 0; y < h; ++y)
        for (uint32_t x = 0; x < w; ++x) {
            const double u = ((double(x) + 0.5) / double(w) * 2.0 - 1.0) * tw;
            const double v = ((double(y) + 0.5) / double(h) * 2.0 - 1.0) * th;
            const d3 d = unit(dir + (U * u + V * v));
            float *r = rays8 + 8 * ((size_t)y * w + x);
            r[0] = (float)pos.x, r[1] = (float)pos.y, r[2] = (float)pos.z, r[3] = tmin;
            r[4] = (float)d.x, r[5] = (float)d.y, r[6] = (float)d.z, r[7] = FLT_MAX;
        }
    return 0;
}

// Camera rays as the reference's cam_ray (libgi/camera.cpp:11-28) computes them, in float:
// U = normalize(cross(dir, up)), V = normalize(cross(U, dir)), u = ((x + 0.5 + off.x) / w * 2 - 1)
// near_w, v likewise, d = normalize((dir + U u) + V v) with normalize(a) = a * (1 / sqrt(a . a)),
// origin pos, t_min = 1e-4 (ray::eps, libgi/rt.h:25), t_max = FLT_MAX. Offsets: offsets2 (two
// floats per pixel), or with jitter != 0 two PCG32 uniform floats minus 0.5 from the stream of
// sequence seed + pixel index, or zero. The file is compiled with -ffp-contract=off, so every
// float operation rounds as written.
void orc_cam_rays(const float *pos3, const float *dir3, const float *up3, float near_w, float near_h, uint32_t w,
                  uint32_t h, const float *offsets2, int jitter, uint64_t seed, float *rays8) {
    struct f3 {
        float x, y, z;
    };
    auto cross = [](f3 a, f3 b) -> f3 {
        return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
    };
    auto norm = [](f3 a) -> f3 {
        const float k = 1.0f / std::sqrt((a.x * a.x + a.y * a.y) + a.z * a.z);
        return {a.x * k, a.y * k, a.z * k};
    };
    const f3 dir = {dir3[0], dir3[1], dir3[2]}, up = {up3[0], up3[1], up3[2]};
    const f3 U = norm(cross(dir, up));
    const f3 V = norm(cross(U, dir));
    for (uint32_t y = 0; y < h; ++y)
        for (uint32_t x = 0; x < w; ++x) {
            const uint64_t i = (uint64_t)y * w + x;
            float ox = 0.0f, oy = 0.0f;
            if (offsets2) {
                ox = offsets2[2 * i];
                oy = offsets2[2 * i + 1];
            } else if (jitter) {
                pcg rng(seed + i);
                const uint32_t a = rng.step(), b = rng.step();
                const float fa = (float)a * 0x1p-32f, fb = (float)b * 0x1p-32f;
                ox = (fa < 0x1.fffffep-1f ? fa : 0x1.fffffep-1f) - 0.5f;
                oy = (fb < 0x1.fffffep-1f ? fb : 0x1.fffffep-1f) - 0.5f;
            }
            const float u = near_w * ((((float)x + 0.5f) + ox) / (float)w * 2.0f - 1.0f);
            const float v = near_h * ((((float)y + 0.5f) + oy) / (float)h * 2.0f - 1.0f);
            const f3 d = norm({(dir.x + U.x * u) + V.x * v, (dir.y + U.y * u) + V.y * v, (dir.z + U.z * u) + V.z * v});
            float *r = rays8 + 8 * i;
            r[0] = pos3[0], r[1] = pos3[1], r[2] = pos3[2], r[3] = 1e-4f;
            r[4] = d.x, r[5] = d.y, r[6] = d.z, r[7] = FLT_MAX;
        }
}

}  // extern "C"
