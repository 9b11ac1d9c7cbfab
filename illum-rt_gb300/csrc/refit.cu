// Refit: new vertex positions for a built tree, the same topology.
//
// The reference rebuilds its BVH for every change of the scene (rt/cuda/base.cpp:88-117). For
// small per-step changes of a mesh (the gradient steps of a differentiable renderer) the
// topology can stay and only the boxes follow the vertices:
//   1. every triangle record is recomputed from the new vertices with the builders' arithmetic
//      (v0 and the rounded differences v0 - v1, v0 - v2), keeping its triangle and material;
//   2. the boxes are fitted bottom-up: one thread starts at every inner node whose two children
//      are leaves, writes the leaves' boxes (min / max over their triangles' vertices) into the
//      node's child records, then climbs: it writes the node's box into its parent's child
//      record and counts itself in at the parent with an atomic; the thread that completes a
//      parent (the last of its inner children to arrive) continues with it. No thread waits for
//      another, and each climb is bounded by the tree depth.
// A box is the exact min / max of its triangles' coordinates, so refitting a tree built without
// early split clipping to unchanged vertices gives back its boxes bit for bit; clipped boxes of
// a tree built with it become the full triangle boxes (larger, so no hit is lost).
#include <cfloat>

#include "refit.hpp"

namespace grt {

namespace {

constexpr int kThreads = 256;
constexpr int kMaxClimb = 128;

inline unsigned blocks_for(uint32_t n) { return (n + kThreads - 1) / kThreads; }

// 1. records: v0 + triangle id, v0 - v1 + material id, v0 - v2
__global__ void __launch_bounds__(kThreads) k_refit_records(const float4 *__restrict__ vpos, const uint4 *__restrict__ tris,
                                                            uint32_t nv, uint32_t nt, float4 *records, uint32_t n,
                                                            unsigned *flags) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    float4 *r = records + 3 * (size_t)k;
    const uint32_t prim = __float_as_uint(r[0].w);
    if (prim >= nt) {
        atomicOr(flags, kRefitBadTree);
        return;
    }
    const uint4 t = tris[prim];
    if (t.x >= nv || t.y >= nv || t.z >= nv) {
        atomicOr(flags, kRefitBadTree);
        return;
    }
    const float4 a = vpos[t.x], b = vpos[t.y], c = vpos[t.z];
    r[0] = make_float4(a.x, a.y, a.z, __uint_as_float(prim));
    r[1] = make_float4(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z), __uint_as_float(t.w));
    r[2] = make_float4(__fsub_rn(a.x, c.x), __fsub_rn(a.y, c.y), __fsub_rn(a.z, c.z), 0.f);
}

// whether every vertex coordinate is finite (the traversal's plain slab test relies on it)
__global__ void __launch_bounds__(kThreads) k_refit_finite(const float4 *__restrict__ vpos, uint32_t nv,
                                                           unsigned *flags) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const float4 v = vpos[i];
    if (!isfinite(v.x) || !isfinite(v.y) || !isfinite(v.z)) atomicOr(flags, kRefitNonFinite);
}

struct box3 {
    float lx, ly, lz, hx, hy, hz;
};

__device__ __forceinline__ void grow(box3 &b, float4 p) {
    b.lx = fminf(b.lx, p.x);
    b.ly = fminf(b.ly, p.y);
    b.lz = fminf(b.lz, p.z);
    b.hx = fmaxf(b.hx, p.x);
    b.hy = fmaxf(b.hy, p.y);
    b.hz = fmaxf(b.hz, p.z);
}

// the box of a leaf: its triangles' vertices (records hold the triangle ids); indices outside
// the arrays flag a malformed tree and are skipped
__device__ box3 leaf_box(int32_t ref, const float4 *__restrict__ records, uint32_t n_records,
                         const uint4 *__restrict__ tris, uint32_t nt, const float4 *__restrict__ vpos, uint32_t nv,
                         unsigned *flags) {
    const uint32_t v = ~(uint32_t)ref;
    const uint32_t first = v >> 4, count = (v & 15u) + 1u;
    box3 b = {FLT_MAX, FLT_MAX, FLT_MAX, -FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (uint32_t k = 0; k < count; ++k) {
        const uint32_t rec = first + k;
        const uint32_t prim = rec < n_records ? __float_as_uint(records[3 * (size_t)rec].w) : nt;
        if (prim >= nt) {
            atomicOr(flags, kRefitBadTree);
            continue;
        }
        const uint4 t = tris[prim];
        if (t.x >= nv || t.y >= nv || t.z >= nv) {
            atomicOr(flags, kRefitBadTree);
            continue;
        }
        grow(b, vpos[t.x]);
        grow(b, vpos[t.y]);
        grow(b, vpos[t.z]);
    }
    return b;
}

// a child record of a binary node: (lo.x, lo.y, hi.x, hi.y), (lo.z, hi.z, ref, 0)
__device__ __forceinline__ void put(float4 *q, int side, const box3 &b, int32_t ref) {
    q[2 * side] = make_float4(b.lx, b.ly, b.hx, b.hy);
    q[2 * side + 1] = make_float4(b.lz, b.hz, __int_as_float(ref), 0.f);
}

// 2. boxes bottom-up
__global__ void __launch_bounds__(kThreads) k_refit_climb(float4 *nodes, const int32_t *__restrict__ links, int32_t root,
                                                          uint32_t n_nodes, const float4 *__restrict__ records,
                                                          uint32_t n_records, const uint4 *__restrict__ tris,
                                                          uint32_t nt, const float4 *__restrict__ vpos, uint32_t nv,
                                                          unsigned *arrive, unsigned *flags) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_nodes) return;
    if ((int32_t)i != root && links[i] < 0) return;  // not a node of the tree
    const int32_t c0 = __float_as_int(nodes[4 * (size_t)i + 1].z), c1 = __float_as_int(nodes[4 * (size_t)i + 3].z);
    if (c0 >= 0 || c1 >= 0) return;  // the climbs start at nodes with two leaf children
    uint32_t node = i;
    for (int step = 0; step < kMaxClimb; ++step) {
        float4 *q = nodes + 4 * (size_t)node;
        box3 b[2];
        for (int side = 0; side < 2; ++side) {
            const int32_t ref = __float_as_int(q[2 * side + 1].z);  // references never change
            if (ref < 0) {
                b[side] = leaf_box(ref, records, n_records, tris, nt, vpos, nv, flags);
                put(q, side, b[side], ref);
            } else {  // written by the thread that completed that child, before its atomic
                const float4 xy = __ldcg(q + 2 * side), z = __ldcg(q + 2 * side + 1);
                b[side] = {xy.x, xy.y, z.x, xy.z, xy.w, z.y};
            }
        }
        const box3 u = {fminf(b[0].lx, b[1].lx), fminf(b[0].ly, b[1].ly), fminf(b[0].lz, b[1].lz),
                        fmaxf(b[0].hx, b[1].hx), fmaxf(b[0].hy, b[1].hy), fmaxf(b[0].hz, b[1].hz)};
        if ((int32_t)node == root) return;
        const int32_t link = links[node];
        const uint32_t p = (uint32_t)link >> 1;
        if (link < 0 || p >= n_nodes) {
            atomicOr(flags, kRefitBadTree);
            return;
        }
        float4 *pq = nodes + 4 * (size_t)p;
        const int side = link & 1;
        put(pq, side, u, (int32_t)node);
        __threadfence();
        const int inner = (__float_as_int(pq[1].z) >= 0) + (__float_as_int(pq[3].z) >= 0);
        if ((int)atomicAdd(arrive + p, 1u) + 1 < inner) return;  // the other child's climb continues
        __threadfence();
        node = p;
    }
    atomicOr(flags, kRefitBadTree);
}

}  // namespace

cudaError_t launch_refit(const refit_args &a, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(a.flags, 0, sizeof(unsigned), st);
    if (e == cudaSuccess && a.n_nodes) e = cudaMemsetAsync(a.arrive, 0, (size_t)a.n_nodes * sizeof(unsigned), st);
    if (e != cudaSuccess) return e;
    if (a.nv) k_refit_finite<<<blocks_for(a.nv), kThreads, 0, st>>>(a.vpos, a.nv, a.flags);
    if (a.n_records)
        k_refit_records<<<blocks_for(a.n_records), kThreads, 0, st>>>(a.vpos, a.tris, a.nv, a.nt, a.records,
                                                                     a.n_records, a.flags);
    if (a.n_nodes)
        k_refit_climb<<<blocks_for(a.n_nodes), kThreads, 0, st>>>(a.nodes, a.links, a.root, a.n_nodes, a.records,
                                                                 a.n_records, a.tris, a.nt, a.vpos, a.nv, a.arrive,
                                                                 a.flags);
    return cudaGetLastError();
}

}  // namespace grt
