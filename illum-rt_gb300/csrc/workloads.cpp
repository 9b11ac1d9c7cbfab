// Seeded synthetic scenes and ray batches for the benchmark and the parity tests.
//
// No scene files ship with the reference (its scripts load render-data/ models that are not
// available), so every workload is generated here from a seed. Output must be bit-identical on
// x86-64 and aarch64: randomness is PCG32 (O'Neill 2014, the same generator the reference
// uses in libgi/random.h:59-96), transcendental functions come from pmath.hpp, and the file is
// compiled with -ffp-contract=off.
//
// Layouts match the reference's CUDA scene upload (rt/cuda/base.cpp:48-68): vertex positions
// as float4 (x, y, z, 1) and triangles as uint4 (a, b, c, material). Rays use the CUDA raydata
// layout (rt/cuda/base.h:337, rt/cuda/kernels.cu:52-60): two float4 per ray,
// (o.x, o.y, o.z, t_min) and (d.x, d.y, d.z, t_max).
#include "pmath.hpp"

#include <cfloat>
#include <cstdint>
#include <cstring>
#include <map>
#include <utility>
#include <vector>

namespace {

struct pcg32 {
    uint64_t state, inc;
    explicit pcg32(uint64_t seq, uint64_t seed = 0x853c49e6748fea9bULL) {
        state = 0;
        inc = (seq << 1u) | 1u;
        next();
        state += seed;
        next();
    }
    uint32_t next() {
        uint64_t old = state;
        state = old * 6364136223846793005ULL + inc;
        uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
        uint32_t rot = (uint32_t)(old >> 59u);
        return (xs >> rot) | (xs << ((32u - rot) & 31u));
    }
    // uniform double in [0, 1) with 53 random bits
    double uniform() {
        uint64_t hi = next() >> 5, lo = next() >> 6;
        return double(hi * 67108864ull + lo) * (1.0 / 9007199254740992.0);
    }
    // standard normal deviate (Box-Muller, one value per call)
    double normal() {
        double u1 = uniform(), u2 = uniform();
        if (u1 < 1e-300) u1 = 1e-300;
        double r = std::sqrt(-2.0 * grt_pm::log(u1));
        return r * grt_pm::cos(2.0 * grt_pm::PI * u2);
    }
};

struct d3 {
    double x, y, z;
};
inline d3 sub(d3 a, d3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline d3 add(d3 a, d3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline d3 mul(d3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline double dot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline d3 cross(d3 a, d3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline d3 normalize(d3 a) { return mul(a, 1.0 / std::sqrt(dot(a, a))); }

inline void put_v(float *v4, uint32_t i, d3 p) {
    v4[4 * i + 0] = (float)p.x;
    v4[4 * i + 1] = (float)p.y;
    v4[4 * i + 2] = (float)p.z;
    v4[4 * i + 3] = 1.0f;
}
inline void put_t(uint32_t *t4, uint32_t i, uint32_t a, uint32_t b, uint32_t c, uint32_t m) {
    t4[4 * i + 0] = a;
    t4[4 * i + 1] = b;
    t4[4 * i + 2] = c;
    t4[4 * i + 3] = m;
}
inline void put_ray(float *r8, uint64_t i, d3 o, d3 d, float tmin, float tmax) {
    float *r = r8 + 8 * i;
    r[0] = (float)o.x;
    r[1] = (float)o.y;
    r[2] = (float)o.z;
    r[3] = tmin;
    r[4] = (float)d.x;
    r[5] = (float)d.y;
    r[6] = (float)d.z;
    r[7] = tmax;
}

}  // namespace

extern "C" {

// Heightfield: n x n vertex grid over [0,1]^2 with z ~ U[0, zmax], two triangles per cell,
// 2 (n-1)^2 triangles. n = 64 gives 4,096 vertices and 7,938 triangles.
void wl_heightfield(uint64_t seed, uint32_t n, float zmax, float *vpos4, uint32_t *tris4) {
    pcg32 rng(seed);
    for (uint32_t j = 0; j < n; ++j)
        for (uint32_t i = 0; i < n; ++i)
            put_v(vpos4, j * n + i, {double(i) / double(n - 1), double(j) / double(n - 1), rng.uniform() * zmax});
    uint32_t t = 0;
    for (uint32_t j = 0; j + 1 < n; ++j)
        for (uint32_t i = 0; i + 1 < n; ++i) {
            uint32_t a = j * n + i, b = a + 1, c = a + n, d = c + 1;
            put_t(tris4, t++, a, b, d, 0);
            put_t(tris4, t++, a, d, c, 0);
        }
}

// `count` UV spheres of `slices` x `stacks` quads, two triangles per quad. The pole rows hold
// `slices` coincident vertices, so each sphere carries 2*slices zero-area triangles, as a mesh
// exported from a modelling tool would. Centres ~ U[-cext, cext]^3, radii ~ U[rmin, rmax].
// Vertices per sphere: (stacks+1)*slices; triangles: 2*slices*stacks.
void wl_spheres(uint64_t seed, uint32_t count, uint32_t slices, uint32_t stacks, float cext, float rmin,
                float rmax, float *vpos4, uint32_t *tris4) {
    pcg32 rng(seed);
    const uint32_t vps = (stacks + 1) * slices, tps = 2 * slices * stacks;
    std::vector<double> st(stacks + 1), ct(stacks + 1), sp(slices), cp(slices);
    for (uint32_t i = 0; i <= stacks; ++i) grt_pm::sincos(grt_pm::PI * double(i) / double(stacks), &st[i], &ct[i]);
    for (uint32_t j = 0; j < slices; ++j) grt_pm::sincos(2.0 * grt_pm::PI * double(j) / double(slices), &sp[j], &cp[j]);
    for (uint32_t s = 0; s < count; ++s) {
        d3 c = {(2 * rng.uniform() - 1) * cext, (2 * rng.uniform() - 1) * cext, (2 * rng.uniform() - 1) * cext};
        double r = rmin + (rmax - rmin) * rng.uniform();
        for (uint32_t i = 0; i <= stacks; ++i)
            for (uint32_t j = 0; j < slices; ++j) {
                // the pole rows use sin(theta) = 0 exactly, so all their vertices coincide
                double sti = (i == 0 || i == stacks) ? 0.0 : st[i];
                double cti = (i == 0) ? 1.0 : (i == stacks ? -1.0 : ct[i]);
                d3 p = {c.x + r * sti * cp[j], c.y + r * cti, c.z + r * sti * sp[j]};
                put_v(vpos4, s * vps + i * slices + j, p);
            }
        for (uint32_t i = 0; i < stacks; ++i)
            for (uint32_t j = 0; j < slices; ++j) {
                uint32_t jn = (j + 1) % slices;
                uint32_t a = s * vps + i * slices + j, b = s * vps + i * slices + jn;
                uint32_t cc = s * vps + (i + 1) * slices + j, d = s * vps + (i + 1) * slices + jn;
                uint32_t t = s * tps + 2 * (i * slices + j);
                put_t(tris4, t, a, cc, d, s);
                put_t(tris4, t + 1, a, d, b, s);
            }
    }
}

// Random triangle soup: centroids ~ U[0,1]^3 * n^(1/3), the two edge vectors ~ N(0, sigma^2)^3.
void wl_soup(uint64_t seed, uint32_t ntri, float sigma, float *vpos4, uint32_t *tris4) {
    pcg32 rng(seed);
    const double scale = grt_pm::cbrt(double(ntri));
    for (uint32_t t = 0; t < ntri; ++t) {
        d3 c = {rng.uniform() * scale, rng.uniform() * scale, rng.uniform() * scale};
        d3 e1 = {rng.normal() * sigma, rng.normal() * sigma, rng.normal() * sigma};
        d3 e2 = {rng.normal() * sigma, rng.normal() * sigma, rng.normal() * sigma};
        d3 v0 = sub(c, mul(add(e1, e2), 1.0 / 3.0));
        put_v(vpos4, 3 * t + 0, v0);
        put_v(vpos4, 3 * t + 1, add(v0, e1));
        put_v(vpos4, 3 * t + 2, add(v0, e2));
        put_t(tris4, t, 3 * t, 3 * t + 1, 3 * t + 2, 0);
    }
}

// Rays for a soup scene: origins uniform on the bounding sphere of the box [lo, hi], each
// aimed at a point uniform inside the box.
void wl_sphere_shell_rays(uint64_t seed, const float *lo3, const float *hi3, uint64_t nrays, float tmin,
                          float *rays8) {
    pcg32 rng(seed);
    d3 lo = {lo3[0], lo3[1], lo3[2]}, hi = {hi3[0], hi3[1], hi3[2]};
    d3 ctr = mul(add(lo, hi), 0.5);
    double rad = 0.5 * std::sqrt(dot(sub(hi, lo), sub(hi, lo)));
    for (uint64_t i = 0; i < nrays; ++i) {
        double z = 2 * rng.uniform() - 1, phi = 2 * grt_pm::PI * rng.uniform();
        double rxy = std::sqrt(1 - z * z);
        d3 u = {rxy * grt_pm::cos(phi), rxy * grt_pm::sin(phi), z};
        d3 o = add(ctr, mul(u, rad));
        d3 tgt = {lo.x + (hi.x - lo.x) * rng.uniform(), lo.y + (hi.y - lo.y) * rng.uniform(),
                  lo.z + (hi.z - lo.z) * rng.uniform()};
        put_ray(rays8, i, o, normalize(sub(tgt, o)), tmin, FLT_MAX);
    }
}

// Log-uniform integer in [lo, hi] (inclusive), e.g. triangle or ray counts of the multi-scene batch.
uint64_t wl_log_uniform(uint64_t seed, uint64_t seq, uint64_t lo, uint64_t hi) {
    pcg32 rng(seed * 0x9E3779B97F4A7C15ull + seq);
    double l = grt_pm::log(double(lo)), h = grt_pm::log(double(hi));
    double v = grt_pm::exp(l + (h - l) * rng.uniform());
    uint64_t r = (uint64_t)std::nearbyint(v);
    return r < lo ? lo : (r > hi ? hi : r);
}

// Icosphere: the regular icosahedron subdivided `levels` times (each triangle into four, new
// vertices projected to the unit sphere), then every vertex displaced radially by
// (1 + disp * N(0,1)). Vertices: 10*4^levels + 2; triangles: 20*4^levels.
void wl_icosphere(uint64_t seed, uint32_t levels, float disp, float *vpos4, uint32_t *tris4) {
    const double g = (1.0 + std::sqrt(5.0)) / 2.0;
    std::vector<d3> v = {{-1, g, 0}, {1, g, 0}, {-1, -g, 0}, {1, -g, 0}, {0, -1, g}, {0, 1, g},
                         {0, -1, -g}, {0, 1, -g}, {g, 0, -1}, {g, 0, 1}, {-g, 0, -1}, {-g, 0, 1}};
    for (auto &p : v) p = normalize(p);
    std::vector<uint32_t> f = {0, 11, 5, 0, 5, 1, 0, 1, 7, 0, 7, 10, 0, 10, 11, 1, 5, 9, 5, 11, 4,
                               11, 10, 2, 10, 7, 6, 7, 1, 8, 3, 9, 4, 3, 4, 2, 3, 2, 6, 3, 6, 8,
                               3, 8, 9, 4, 9, 5, 2, 4, 11, 6, 2, 10, 8, 6, 7, 9, 8, 1};
    for (uint32_t l = 0; l < levels; ++l) {
        std::map<std::pair<uint32_t, uint32_t>, uint32_t> mid;
        auto midpoint = [&](uint32_t a, uint32_t b) {
            auto key = a < b ? std::make_pair(a, b) : std::make_pair(b, a);
            auto it = mid.find(key);
            if (it != mid.end()) return it->second;
            uint32_t id = (uint32_t)v.size();
            v.push_back(normalize(mul(add(v[a], v[b]), 0.5)));
            mid[key] = id;
            return id;
        };
        std::vector<uint32_t> nf;
        nf.reserve(f.size() * 4);
        for (size_t i = 0; i < f.size(); i += 3) {
            uint32_t a = f[i], b = f[i + 1], c = f[i + 2];
            uint32_t ab = midpoint(a, b), bc = midpoint(b, c), ca = midpoint(c, a);
            uint32_t add4[12] = {a, ab, ca, b, bc, ab, c, ca, bc, ab, bc, ca};
            nf.insert(nf.end(), add4, add4 + 12);
        }
        f.swap(nf);
    }
    pcg32 rng(seed);
    for (uint32_t i = 0; i < v.size(); ++i) put_v(vpos4, i, mul(v[i], 1.0 + disp * rng.normal()));
    for (uint32_t t = 0; t < f.size() / 3; ++t) put_t(tris4, t, f[3 * t], f[3 * t + 1], f[3 * t + 2], 0);
}

// Pinhole camera rays, pixel centres, in the construction of the reference's cam_ray
// (libgi/camera.cpp:11-28; frustum from libgi/camera.h:18-24): U = normalize(dir x up),
// V = normalize(U x dir), u,v in (-1,1) scaled by the near-plane half extents,
// d = normalize(dir + u U + v V). Computed in double and rounded once to float, so the same
// rays come out on every host. Ray (x, y) is stored at index y*w + x.
void wl_camera_rays(const float *pos3, const float *look3, const float *up3, float fovy_deg, uint32_t w,
                    uint32_t h, float tmin, float *rays8) {
    d3 pos = {pos3[0], pos3[1], pos3[2]}, look = {look3[0], look3[1], look3[2]}, up = {up3[0], up3[1], up3[2]};
    d3 dir = normalize(sub(look, pos));
    d3 U = normalize(cross(dir, up));
    d3 V = normalize(cross(U, dir));
    double near_h = grt_pm::tan(grt_pm::PI * double(fovy_deg) * 0.5 / 180.0);
    double near_w = near_h * double(w) / double(h);
    for (uint32_t y = 0; y < h; ++y)
        for (uint32_t x = 0; x < w; ++x) {
            double u = ((double(x) + 0.5) / double(w) * 2.0 - 1.0) * near_w;
            double vv = ((double(y) + 0.5) / double(h) * 2.0 - 1.0) * near_h;
            d3 d = normalize(add(dir, add(mul(U, u), mul(V, vv))));
            put_ray(rays8, uint64_t(y) * w + x, pos, d, tmin, FLT_MAX);
        }
}

// Standard normal float deviates (loss weights and per-vertex scalars of the adjoint workload).
void wl_normals(uint64_t seed, uint64_t n, float *out) {
    pcg32 rng(seed);
    for (uint64_t i = 0; i < n; ++i) out[i] = (float)rng.normal();
}

}  // extern "C"
