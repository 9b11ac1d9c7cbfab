// Camera rays of the primary-ray step (grt_camera_rays; cam_ray, libgi/camera.cpp:11-28, in its
// own float arithmetic), and incoherent test rays: the reference CUDA tracer's
// `incoherence r1 r2` setting
// (rt/cuda/base.cpp:120-133), which replaces the camera rays by rays between two spheres placed
// in the scene (batch_cam_ray_setup::run, rt/cuda/rni.cpp:36-84; setup_ray_incoherent,
// rt/cuda/kernels.cu:75-156):
//   * the scene's extent is the bounding box of its vertices; along its largest dimension the
//     two sphere centres sit at the quarter points, centred in the other two, and r_max is a
//     quarter of that dimension;
//   * a ray starts at a uniform point in the ball of radius r1 * r_max around the first centre
//     (the centre itself for r1 = 0) and aims at a uniform point in the ball of radius
//     r2 * r_max around the second (its centre for r2 = 0): phi = 2 pi u1, cos(theta) = 2 u2 - 1,
//     r = radius * cbrt(u3); t_min 0, t_max FLT_MAX.
// Differences: the uniform numbers come from a PCG32 stream per ray (seed + ray index) instead
// of cuRAND's MTGP32 generator, the direction is normalised as v * (1 / sqrt(v . v)) with
// rounded operations, and the trigonometric and cube-root functions are CUDA's.
#include <cfloat>

#include "pt_math.cuh"
#include "raygen.hpp"

namespace grt {

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ uint32_t ordered(float f) {
    const uint32_t b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float unordered(uint32_t u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

// bounds[0..2] = min xyz, bounds[3..5] = max xyz, as order-preserving integers
__global__ void __launch_bounds__(kThreads) k_extent(const float4 *__restrict__ vpos, uint32_t nv, uint32_t *bounds) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const float4 v = vpos[i];
    atomicMin(bounds + 0, ordered(v.x));
    atomicMin(bounds + 1, ordered(v.y));
    atomicMin(bounds + 2, ordered(v.z));
    atomicMax(bounds + 3, ordered(v.x));
    atomicMax(bounds + 4, ordered(v.y));
    atomicMax(bounds + 5, ordered(v.z));
}

struct spheres2 {
    pm::f3 c1, c2;
    float r_max;
};

// the sphere placement of batch_cam_ray_setup::run (rt/cuda/rni.cpp:38-66)
__device__ spheres2 place(const uint32_t *bounds) {
    const pm::f3 lo = {unordered(bounds[0]), unordered(bounds[1]), unordered(bounds[2])};
    const pm::f3 hi = {unordered(bounds[3]), unordered(bounds[4]), unordered(bounds[5])};
    const pm::f3 sz = {fabsf(pm::sub(hi.x, lo.x)), fabsf(pm::sub(hi.y, lo.y)), fabsf(pm::sub(hi.z, lo.z))};
    const pm::f3 mid = {pm::add(lo.x, pm::div(sz.x, 2.f)), pm::add(lo.y, pm::div(sz.y, 2.f)),
                        pm::add(lo.z, pm::div(sz.z, 2.f))};
    spheres2 s;
    s.c1 = s.c2 = mid;
    if (sz.x >= sz.y && sz.x >= sz.z) {
        s.r_max = pm::div(sz.x, 4.f);
        s.c1.x = pm::add(lo.x, s.r_max);
        s.c2.x = pm::sub(hi.x, s.r_max);
    } else if (sz.y >= sz.x && sz.y >= sz.z) {
        s.r_max = pm::div(sz.y, 4.f);
        s.c1.y = pm::add(lo.y, s.r_max);
        s.c2.y = pm::sub(hi.y, s.r_max);
    } else {
        s.r_max = pm::div(sz.z, 4.f);
        s.c1.z = pm::add(lo.z, s.r_max);
        s.c2.z = pm::sub(hi.z, s.r_max);
    }
    return s;
}

// a uniform point in the ball of radius `radius` (setup_ray_incoherent's sampling)
__device__ pm::f3 in_ball(pm::pcg32 &rng, float radius) {
    const float u1 = rng.uniform(), u2 = rng.uniform(), u3 = rng.uniform();
    const float phi = pm::mul(pm::mul(u1, 2.f), 3.14159265358979323846f);
    const float cos_t = pm::sub(pm::mul(u2, 2.f), 1.f);
    const float theta = acosf(cos_t);
    const float r = pm::mul(radius, cbrtf(u3));
    float st, ct, sp, cp;
    sincosf(theta, &st, &ct);
    sincosf(phi, &sp, &cp);
    return {pm::mul(pm::mul(r, st), cp), pm::mul(pm::mul(r, st), sp), pm::mul(r, ct)};
}

__global__ void __launch_bounds__(kThreads) k_incoherent(const uint32_t *__restrict__ bounds, float r1, float r2,
                                                         uint64_t seed, float4 *rays, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const spheres2 sp = place(bounds);
    pm::pcg32 rng;
    rng.set_sequence(seed + i);
    pm::f3 o = sp.c1;
    if (r1 > 0.f) {
        const pm::f3 q = in_ball(rng, pm::mul(r1, sp.r_max));
        o = {pm::add(o.x, q.x), pm::add(o.y, q.y), pm::add(o.z, q.z)};
    }
    pm::f3 target = sp.c2;
    if (r2 > 0.f) {
        const pm::f3 q = in_ball(rng, pm::mul(r2, sp.r_max));
        target = {pm::add(target.x, q.x), pm::add(target.y, q.y), pm::add(target.z, q.z)};
    }
    const pm::f3 d = pm::normalize3(pm::sub3(target, o));
    rays[2 * (size_t)i] = make_float4(o.x, o.y, o.z, 0.f);
    rays[2 * (size_t)i + 1] = make_float4(d.x, d.y, d.z, FLT_MAX);
}

// The camera of the primary-ray step, by value.
struct cam_t {
    pm::f3 pos, dir, up;
    float near_w, near_h;
};

// cam_ray (libgi/camera.cpp:11-28) for pixel i = y w + x, every operation rounded as the float
// code rounds it (glm's normalize is a * (1 / sqrt(dot(a, a))), its dot ((x x' + y y') + z z'),
// its cross (a.y b.z - b.y a.z, a.z b.x - b.z a.x, a.x b.y - b.x a.y)). One thread per ray;
// the 32-byte ray is written with two 16-byte stores.
__global__ void __launch_bounds__(kThreads) k_camera_rays(cam_t cam, uint32_t w, uint32_t h,
                                                          const float2 *__restrict__ offsets, int jitter,
                                                          uint64_t seed, float4 *rays) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (uint64_t)w * h) return;
    const uint32_t y = (uint32_t)(i / w), x = (uint32_t)(i - (uint64_t)y * w);
    auto cross = [](pm::f3 a, pm::f3 b) -> pm::f3 {
        return {pm::sub(pm::mul(a.y, b.z), pm::mul(b.y, a.z)), pm::sub(pm::mul(a.z, b.x), pm::mul(b.z, a.x)),
                pm::sub(pm::mul(a.x, b.y), pm::mul(b.x, a.y))};
    };
    const pm::f3 U = pm::normalize3(cross(cam.dir, cam.up));
    const pm::f3 V = pm::normalize3(cross(U, cam.dir));
    float ox = 0.f, oy = 0.f;
    if (offsets) {
        const float2 o = offsets[i];
        ox = o.x;
        oy = o.y;
    } else if (jitter) {
        pm::pcg32 rng;
        rng.set_sequence(seed + i);
        ox = pm::sub(rng.uniform(), 0.5f);
        oy = pm::sub(rng.uniform(), 0.5f);
    }
    const float u = pm::mul(cam.near_w, pm::sub(pm::mul(pm::div(pm::add(pm::add((float)x, 0.5f), ox), (float)w), 2.0f), 1.0f));
    const float v = pm::mul(cam.near_h, pm::sub(pm::mul(pm::div(pm::add(pm::add((float)y, 0.5f), oy), (float)h), 2.0f), 1.0f));
    const pm::f3 d = pm::normalize3({pm::add(pm::add(cam.dir.x, pm::mul(U.x, u)), pm::mul(V.x, v)),
                                     pm::add(pm::add(cam.dir.y, pm::mul(U.y, u)), pm::mul(V.y, v)),
                                     pm::add(pm::add(cam.dir.z, pm::mul(U.z, u)), pm::mul(V.z, v))});
    rays[2 * i] = make_float4(cam.pos.x, cam.pos.y, cam.pos.z, 1e-4f);
    rays[2 * i + 1] = make_float4(d.x, d.y, d.z, FLT_MAX);
}

}  // namespace

cudaError_t launch_camera_rays(const float c[11], uint32_t w, uint32_t h, const float2 *offsets, bool jitter,
                               uint64_t seed, float4 *rays, cudaStream_t st) {
    const uint64_t n = (uint64_t)w * h;
    if (n == 0) return cudaSuccess;
    cam_t cam = {{c[0], c[1], c[2]}, {c[3], c[4], c[5]}, {c[6], c[7], c[8]}, c[9], c[10]};
    k_camera_rays<<<(unsigned)((n + kThreads - 1) / kThreads), kThreads, 0, st>>>(cam, w, h, offsets, jitter ? 1 : 0,
                                                                                 seed, rays);
    return cudaGetLastError();
}

cudaError_t launch_incoherent_rays(const float4 *vpos, uint32_t nv, float r1, float r2, uint64_t seed, float4 *rays,
                                   uint32_t n, uint32_t *bounds, cudaStream_t st) {
    // min slots start at the largest key, max slots at the smallest
    cudaError_t e = cudaMemsetAsync(bounds, 0xff, 3 * sizeof(uint32_t), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(bounds + 3, 0, 3 * sizeof(uint32_t), st);
    if (e != cudaSuccess) return e;
    if (nv) k_extent<<<(nv + kThreads - 1) / kThreads, kThreads, 0, st>>>(vpos, nv, bounds);
    if (n) k_incoherent<<<(n + kThreads - 1) / kThreads, kThreads, 0, st>>>(bounds, r1, r2, seed, rays, n);
    return cudaGetLastError();
}

}  // namespace grt
