// Adjoint of the closest hit with respect to the triangle's vertices and the ray.
//
// There is no counterpart in the reference. For a ray (o, d) that hit triangle (A, B, C) the
// reference's Cramer system (libgi/intersect.h:36-58) reads
//     M x = j,   M = [A - B | A - C | d] (columns),   x = (beta, gamma, t),   j = A - o.
// Holding the triangle fixed, dx = M^-1 (dj - dM x), so for an upstream gradient g = dL/dx:
//     lambda = M^-T g
//     dL/dA = lambda (1 - beta - gamma),  dL/dB = lambda beta,  dL/dC = lambda gamma,
//     dL/do = -lambda,                    dL/dd = -lambda t.
// M^-T g is evaluated with cross products: for a matrix with rows r0, r1, r2 the inverse has
// columns (r1 x r2, r2 x r0, r0 x r1) / (r0 . (r1 x r2)); here the rows of M^T are A - B, A - C
// and d. The kernel recomputes x from the current vertices instead of reading stored values.
//
// Vertex gradients are scattered with warp-aggregated atomics: lanes whose hits share a vertex
// (common for coherent rays) are grouped with __match_any_sync, each group's sum is formed with
// a warp reduction and added by one leader lane. When a warp's hits are spread over too many
// vertices the lanes add their own contributions directly.
#include <cfloat>

#include "adjoint.hpp"

namespace grt {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kMaxGroups = 6;  // beyond this many distinct vertices per warp, atomics per lane

struct v3f {
    float x, y, z;
};
__device__ __forceinline__ v3f sub(v3f a, v3f b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ v3f cross(v3f a, v3f b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ float dot(v3f a, v3f b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ v3f scale(v3f a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ v3f add(v3f a, v3f b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
    return v;
}

// Adds g to grad[3*key .. 3*key+2] for every lane with key != ~0u, aggregating equal keys.
__device__ __forceinline__ void scatter_vertex(float *grad, uint32_t key, v3f g) {
    const bool want = key != 0xffffffffu;
    const unsigned lane = threadIdx.x & 31u;
    const unsigned peers = __match_any_sync(kFull, key);
    // count distinct keys among the lanes that want to add
    unsigned leaders = __ballot_sync(kFull, want && (__ffs(peers) - 1) == (int)lane);
    if (__popc(leaders) > kMaxGroups) {
        if (want) {
            atomicAdd(grad + 3 * (size_t)key + 0, g.x);
            atomicAdd(grad + 3 * (size_t)key + 1, g.y);
            atomicAdd(grad + 3 * (size_t)key + 2, g.z);
        }
        return;
    }
    while (leaders) {
        const int leader = __ffs(leaders) - 1;
        leaders &= leaders - 1;
        const uint32_t lkey = __shfl_sync(kFull, key, leader);
        const bool mine = want && key == lkey;
        const float sx = warp_sum(mine ? g.x : 0.f);
        const float sy = warp_sum(mine ? g.y : 0.f);
        const float sz = warp_sum(mine ? g.z : 0.f);
        if ((int)lane == leader) {
            atomicAdd(grad + 3 * (size_t)lkey + 0, sx);
            atomicAdd(grad + 3 * (size_t)lkey + 1, sy);
            atomicAdd(grad + 3 * (size_t)lkey + 2, sz);
        }
    }
}

__global__ void __launch_bounds__(256) k_adjoint(const float4 *__restrict__ rays, const grt_hit *__restrict__ hits,
                                                 const float *__restrict__ grad_tbg, uint32_t n,
                                                 const float4 *__restrict__ vpos, uint32_t vstride,
                                                 const uint4 *__restrict__ tris, float *grad_v,
                                                 float4 *grad_rays) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    bool ok = i < n;
    uint4 tri = make_uint4(0xffffffffu, 0xffffffffu, 0xffffffffu, 0);
    v3f dA = {0, 0, 0}, dB = {0, 0, 0}, dC = {0, 0, 0};
    if (ok) {
        const grt_hit h = hits[i];
        ok = h.t != FLT_MAX;
        v3f go = {0, 0, 0}, gd = {0, 0, 0};
        if (ok) {
            tri = __ldg(tris + h.ref);
            const float *vp = reinterpret_cast<const float *>(vpos);
            const v3f A = {vp[vstride * tri.x], vp[vstride * tri.x + 1], vp[vstride * tri.x + 2]};
            const v3f B = {vp[vstride * tri.y], vp[vstride * tri.y + 1], vp[vstride * tri.y + 2]};
            const v3f C = {vp[vstride * tri.z], vp[vstride * tri.z + 1], vp[vstride * tri.z + 2]};
            const float4 ro = rays[2 * (size_t)i], rd = rays[2 * (size_t)i + 1];
            const v3f o = {ro.x, ro.y, ro.z}, d = {rd.x, rd.y, rd.z};
            const v3f e1 = sub(A, B), e2 = sub(A, C), j = sub(A, o);
            const v3f c12 = cross(e2, d), c20 = cross(d, e1), c01 = cross(e1, e2);
            const float det = dot(e1, c12);
            const float inv = 1.0f / det;
            // x = M^-1 j: rows of M^-1 are (e2 x d, d x e1, e1 x e2) / det
            const float beta = dot(c12, j) * inv, gamma = dot(c20, j) * inv, t = dot(c01, j) * inv;
            const float gt = grad_tbg[3 * (size_t)i], gb = grad_tbg[3 * (size_t)i + 1],
                        gg = grad_tbg[3 * (size_t)i + 2];  // (dL/dt, dL/dbeta, dL/dgamma)
            const v3f lambda = scale(add(add(scale(c12, gb), scale(c20, gg)), scale(c01, gt)), inv);
            dA = scale(lambda, 1.0f - beta - gamma);
            dB = scale(lambda, beta);
            dC = scale(lambda, gamma);
            go = scale(lambda, -1.0f);
            gd = scale(lambda, -t);
        }
        if (grad_rays) {
            grad_rays[2 * (size_t)i] = make_float4(go.x, go.y, go.z, 0.f);
            grad_rays[2 * (size_t)i + 1] = make_float4(gd.x, gd.y, gd.z, 0.f);
        }
    }
    if (grad_v) {
        scatter_vertex(grad_v, ok ? tri.x : 0xffffffffu, dA);
        scatter_vertex(grad_v, ok ? tri.y : 0xffffffffu, dB);
        scatter_vertex(grad_v, ok ? tri.z : 0xffffffffu, dC);
    }
}

}  // namespace

cudaError_t launch_adjoint(const float4 *rays, const grt_hit *hits, const float *grad_tbg, uint32_t n,
                           const float4 *vpos, uint32_t vstride, const uint4 *tris, float *grad_v, float4 *grad_rays,
                           cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    const uint32_t blocks = (n + 255) / 256;
    k_adjoint<<<blocks, 256, 0, st>>>(rays, hits, grad_tbg, n, vpos, vstride, tris, grad_v, grad_rays);
    return cudaGetLastError();
}

}  // namespace grt
