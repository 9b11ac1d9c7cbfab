// BVH construction on the GPU.
//
// The reference builds every BVH on the host (rt/cuda/base.cpp:88-117 calls the CPU builder of
// rt/cpu/bvh-ctor.h:371-503); for large or changing scenes that build, not traversal, is the
// cost. This builder is a linear BVH (Karras, "Maximizing parallelism in the construction of
// BVHs, octrees, and k-d trees", HPG 2012):
//   1. per triangle: its box, and the bounds of all box centres (one pass);
//   2. 30-bit Morton codes of the centres in those bounds, radix-sorted with the triangle index
//      as value (a stable sort, so equal codes keep index order);
//   3. the binary radix tree over the sorted codes, one thread per inner node (equal codes are
//      told apart by their positions);
//   4. boxes fitted bottom-up, one thread per leaf climbing while it is the second child to
//      arrive at a node (an atomic counter per node; no thread ever waits for another). On the
//      way up, a subtree of at most `max_leaf` triangles becomes one leaf when the surface-area
//      cost of a leaf, A n, is not above that of keeping the split, A + S_l + S_r (traversal and
//      intersection costs of 1, as in the reference's SAH, rt/cpu/bvh-ctor.h:477-487). Leaves are
//      contiguous ranges of the sorted order, so records are stored in that order;
//   5. the 4-wide tree: the binary inner nodes at even depth, each taking its children's
//      children (the same collapse as flatten_bvh4 on the host).
// Instead of steps 2 and 3, the SAH method (gpu_build_sah.cu) splits top down with the
// reference's SAH rule, and steps 4 and 5 follow as for the others.
// The trees differ from the reference builder's, so closest hits equal the reference's except
// near-ties, as for the speculative tracers.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <algorithm>
#include <cfloat>

#include "gpu_build.hpp"
#include "grt_internal.hpp"

namespace grt {

namespace {

constexpr int kThreads = 256;
constexpr int kMaxClimb = 128;  // a radix tree over 30-bit codes and 2^27 positions is < 60 deep

__device__ __forceinline__ uint32_t ordered(float f) {
    const uint32_t b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float unordered(uint32_t u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

__device__ __forceinline__ uint32_t spread10(uint32_t v) {  // 10 bits -> every third bit of 30
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000ffu;
    v = (v | (v << 8)) & 0x0300f00fu;
    v = (v | (v << 4)) & 0x030c30c3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

__device__ __forceinline__ float half_area(float4 lo, float4 hi) {
    const float dx = hi.x - lo.x, dy = hi.y - lo.y, dz = hi.z - lo.z;
    return dx * dy + dy * dz + dz * dx;
}

// the bound word w of the 12 (centre min, centre max, box min, box max): a minimum?
__device__ __forceinline__ bool bound_is_min(unsigned w) { return w < 3 || (w >= 6 && w < 9); }

// 1. triangle boxes and the bounds of their centres (combined per warp, then per block, so that
// one block adds to the 12 shared bound words once)
__global__ void __launch_bounds__(kThreads) k_prims(const float4 *__restrict__ vpos, uint32_t nv,
                                                    const uint4 *__restrict__ tris, uint32_t nt, float4 *lo_out,
                                                    float4 *hi_out, uint32_t *cbounds, int32_t *info) {
    __shared__ uint32_t s_bounds[12];
    if (threadIdx.x < 12) s_bounds[threadIdx.x] = bound_is_min(threadIdx.x) ? 0xffffffffu : 0u;
    __syncthreads();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    float cmin[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, cmax[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    float bmin[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, bmax[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    if (i < nt) {
        const uint4 t = tris[i];
        float4 lo = make_float4(0.f, 0.f, 0.f, 0.f), hi = lo;
        if (t.x >= nv || t.y >= nv || t.z >= nv) {
            atomicOr(info + GB_ERR, GB_ERR_INDEX);
        } else {
            const float4 a = vpos[t.x], b = vpos[t.y], c = vpos[t.z];
            lo = make_float4(fminf(fminf(a.x, b.x), c.x), fminf(fminf(a.y, b.y), c.y), fminf(fminf(a.z, b.z), c.z), 0.f);
            hi = make_float4(fmaxf(fmaxf(a.x, b.x), c.x), fmaxf(fmaxf(a.y, b.y), c.y), fmaxf(fmaxf(a.z, b.z), c.z), 0.f);
            const bool fin = isfinite(a.x) && isfinite(a.y) && isfinite(a.z) && isfinite(b.x) && isfinite(b.y) &&
                             isfinite(b.z) && isfinite(c.x) && isfinite(c.y) && isfinite(c.z);
            if (!fin) {
                atomicAnd(info + GB_FINITE, 0);
            } else {
                const float cx = 0.5f * (lo.x + hi.x), cy = 0.5f * (lo.y + hi.y), cz = 0.5f * (lo.z + hi.z);
                cmin[0] = cmax[0] = cx;
                cmin[1] = cmax[1] = cy;
                cmin[2] = cmax[2] = cz;
                bmin[0] = lo.x;
                bmin[1] = lo.y;
                bmin[2] = lo.z;
                bmax[0] = hi.x;
                bmax[1] = hi.y;
                bmax[2] = hi.z;
            }
        }
        lo_out[i] = lo;
        hi_out[i] = hi;
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            cmin[a] = fminf(cmin[a], __shfl_xor_sync(0xffffffffu, cmin[a], o));
            cmax[a] = fmaxf(cmax[a], __shfl_xor_sync(0xffffffffu, cmax[a], o));
            bmin[a] = fminf(bmin[a], __shfl_xor_sync(0xffffffffu, bmin[a], o));
            bmax[a] = fmaxf(bmax[a], __shfl_xor_sync(0xffffffffu, bmax[a], o));
        }
    }
    if ((threadIdx.x & 31u) == 0 && cmin[0] <= cmax[0]) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            atomicMin(s_bounds + a, ordered(cmin[a]));
            atomicMax(s_bounds + 3 + a, ordered(cmax[a]));
            atomicMin(s_bounds + 6 + a, ordered(bmin[a]));
            atomicMax(s_bounds + 9 + a, ordered(bmax[a]));
        }
    }
    __syncthreads();
    if (threadIdx.x < 12) {
        const uint32_t v = s_bounds[threadIdx.x];
        if (bound_is_min(threadIdx.x)) {
            if (v != 0xffffffffu) atomicMin(cbounds + threadIdx.x, v);
        } else if (v != 0u) {
            atomicMax(cbounds + threadIdx.x, v);
        }
    }
}

// 2. Morton codes of the box centres
__global__ void __launch_bounds__(kThreads) k_morton(const float4 *__restrict__ lo, const float4 *__restrict__ hi,
                                                     uint32_t n, const uint32_t *__restrict__ cbounds, uint32_t *keys,
                                                     uint32_t *vals) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 l = lo[i], h = hi[i];
    const float c[3] = {0.5f * (l.x + h.x), 0.5f * (l.y + h.y), 0.5f * (l.z + h.z)};
    uint32_t q[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float mn = unordered(cbounds[a]), mx = unordered(cbounds[3 + a]);
        const float ext = mx - mn;
        float u = ext > 0.f ? (c[a] - mn) / ext : 0.f;
        u = fminf(fmaxf(u * 1024.f, 0.f), 1023.f);  // NaN -> 0
        q[a] = (uint32_t)u;
    }
    keys[i] = (spread10(q[0]) << 2) | (spread10(q[1]) << 1) | spread10(q[2]);
    vals[i] = i;
}

// length of the common prefix of the keys at positions i and j (positions break ties)
__device__ __forceinline__ int prefix(const uint32_t *__restrict__ k, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    const uint32_t a = k[i], b = k[j];
    return a != b ? __clz(a ^ b) : 32 + __clz((uint32_t)(i ^ j));
}

// 3. the radix tree: inner node i covers sorted positions [first, last]; children are inner
// nodes (>= 0) or single positions (~pos)
__global__ void __launch_bounds__(kThreads) k_radix_tree(const uint32_t *__restrict__ keys, int n, int2 *children,
                                                         int2 *range, int32_t *parent_inner, int32_t *parent_leaf) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    const int d = prefix(keys, n, i, i + 1) - prefix(keys, n, i, i - 1) >= 0 ? 1 : -1;
    const int dmin = prefix(keys, n, i, i - d);
    int lmax = 2;
    while (prefix(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (prefix(keys, n, i, i + (l + t) * d) > dmin) l += t;
    const int j = i + l * d;
    const int dnode = prefix(keys, n, i, j);
    int s = 0;
    for (int div = 2;; div <<= 1) {
        const int t = (l + div - 1) / div;
        if (prefix(keys, n, i, i + (s + t) * d) > dnode) s += t;
        if (t <= 1) break;
    }
    const int split = i + s * d + (d < 0 ? -1 : 0);
    const int first = min(i, j), last = max(i, j);
    const int left = first == split ? ~split : split;
    const int right = last == split + 1 ? ~(split + 1) : split + 1;
    children[i] = make_int2(left, right);
    range[i] = make_int2(first, last);
    if (left >= 0)
        parent_inner[left] = i;
    else
        parent_leaf[~left] = i;
    if (right >= 0)
        parent_inner[right] = i;
    else
        parent_leaf[~right] = i;
    if (i == 0) parent_inner[0] = -1;
}

// ---- 3'. PLOC: parallel locally-ordered clustering over the Morton order --------------------
//
// After Meister and Bittner, "Parallel Locally-Ordered Clustering for Bounding Volume Hierarchy
// Construction" (IEEE TVCG 2018): the sorted triangles start as clusters; in every iteration
// each cluster finds, among the kPlocRadius clusters on either side of it in the current list,
// the one whose union box has the smallest surface area; mutual nearest neighbours merge into a
// new inner node, and the list is compacted in order. Ties are broken by the nearer list
// position, then by parity (an even position prefers its right neighbour, an odd one its left),
// so that coincident triangles pair up and halve each iteration. After a budget of iterations
// any remaining clusters are paired by position ((0, 1), (2, 3), ...), which bounds the number of
// iterations and the tree's depth. Every index comes from a prefix sum, so the tree is the same
// on every run. Cluster ids: sorted position k for a triangle, n + q for the q-th inner node made.
// The finished tree is renumbered into the radix tree's form (children, ranges and parents, the
// root as inner node 0, leaves as positions of a depth-first order), so the rest of the build
// (bottom-up fit, SAH collapse, records, 4-wide collapse) is shared.

constexpr int kPlocRadius = 16;

struct ploc_state {
    int32_t m;      // clusters in the current list
    int32_t made;   // inner nodes made so far
    int32_t err;    // an index outside its array was met (never for a well-formed run)
    int32_t pad;
};

__global__ void __launch_bounds__(kThreads) k_ploc_init(const float4 *__restrict__ lo, const float4 *__restrict__ hi,
                                                        const uint32_t *__restrict__ order, int n, int32_t *cl,
                                                        float4 *box_lo, float4 *box_hi, int32_t *parent,
                                                        ploc_state *ps) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k == 0) *ps = {n, 0, 0, 0};
    if (k >= n) return;
    const uint32_t prim = order[k];
    cl[k] = k;
    box_lo[k] = lo[prim];
    box_hi[k] = hi[prim];
    parent[k] = -1;
    if (k < n - 1) parent[n + k] = -1;
}

// Nearest neighbour of every cluster (or, when `forced`, its pairing partner). The block's
// clusters and kPlocRadius on either side are staged in shared memory.
__global__ void __launch_bounds__(kThreads) k_ploc_nn(const int32_t *__restrict__ cl,
                                                      const float4 *__restrict__ box_lo,
                                                      const float4 *__restrict__ box_hi,
                                                      const ploc_state *__restrict__ ps, int forced, int32_t *nn) {
    __shared__ float4 s_lo[kThreads + 2 * kPlocRadius], s_hi[kThreads + 2 * kPlocRadius];
    const int m = ps->m;
    const int b0 = blockIdx.x * kThreads;
    if (m <= 1 || b0 >= m) return;
    const int i = b0 + threadIdx.x;
    if (forced) {
        if (i < m) nn[i] = (i ^ 1) < m ? (i ^ 1) : -1;
        return;
    }
    for (int t = threadIdx.x; t < kThreads + 2 * kPlocRadius; t += kThreads) {
        const int g = b0 - kPlocRadius + t;
        if (g >= 0 && g < m) {
            const int id = cl[g];
            s_lo[t] = box_lo[id];
            s_hi[t] = box_hi[id];
        }
    }
    __syncthreads();
    if (i >= m) return;
    const int me = threadIdx.x + kPlocRadius;
    const float4 a_lo = s_lo[me], a_hi = s_hi[me];
    float best = __int_as_float(0x7f800000);
    int bj = -1, bd = 1 << 30;
    const bool even = (i & 1) == 0;
    for (int d = -kPlocRadius; d <= kPlocRadius; ++d) {
        const int j = i + d;
        if (d == 0 || j < 0 || j >= m) continue;
        const float4 b_lo = s_lo[me + d], b_hi = s_hi[me + d];
        const float4 ulo = make_float4(fminf(a_lo.x, b_lo.x), fminf(a_lo.y, b_lo.y), fminf(a_lo.z, b_lo.z), 0.f);
        const float4 uhi = make_float4(fmaxf(a_hi.x, b_hi.x), fmaxf(a_hi.y, b_hi.y), fmaxf(a_hi.z, b_hi.z), 0.f);
        const float area = half_area(ulo, uhi);
        const int ad = d < 0 ? -d : d;
        const bool pref = even ? d > 0 : d < 0;
        if (area < best || (area == best && (ad < bd || (ad == bd && pref)))) {
            best = area;
            bj = j;
            bd = ad;
        }
    }
    nn[i] = bj;
}

// Merge flags: high word 1 for the lower position of a mutual pair (it makes the new node),
// low word 1 for every position that stays in the list (all but the higher one of a pair).
__global__ void __launch_bounds__(kThreads) k_ploc_flags(const int32_t *__restrict__ nn,
                                                         const ploc_state *__restrict__ ps, int n,
                                                         unsigned long long *flags) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int m = ps->m;
    unsigned long long f = 0;
    if (i < m && m > 1) {
        const int j = nn[i];
        const bool mutual = j >= 0 && j < m && nn[j] == i;
        const bool merge = mutual && i < j, drop = mutual && i > j;
        f = ((unsigned long long)(merge ? 1u : 0u) << 32) | (drop ? 0u : 1u);
    } else if (i < m) {
        f = 1;
    }
    flags[i] = f;
}

__global__ void __launch_bounds__(kThreads) k_ploc_apply(const int32_t *__restrict__ cl, const int32_t *__restrict__ nn,
                                                         const unsigned long long *__restrict__ flags,
                                                         const unsigned long long *__restrict__ excl, int n,
                                                         ploc_state *ps, int2 *kid, float4 *box_lo,
                                                         float4 *box_hi, int32_t *parent, int32_t *cl_next) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int m = ps->m;
    if (i >= m || m <= 1) return;
    const unsigned long long f = flags[i], e = excl[i];
    const int keep_pos = (int)(uint32_t)e;
    if (f >> 32) {
        const int j = nn[i];
        const int q = ps->made + (int)(e >> 32);
        if (q < 0 || q >= n - 1 || j < 0 || j >= m) {
            atomicOr(&ps->err, 1);
            return;
        }
        const int a = cl[i], b = cl[j];
        const int id = n + q;
        kid[q] = make_int2(a, b);
        const float4 al = box_lo[a], ah = box_hi[a], bl = box_lo[b], bh = box_hi[b];
        box_lo[id] = make_float4(fminf(al.x, bl.x), fminf(al.y, bl.y), fminf(al.z, bl.z), 0.f);
        box_hi[id] = make_float4(fmaxf(ah.x, bh.x), fmaxf(ah.y, bh.y), fmaxf(ah.z, bh.z), 0.f);
        parent[a] = q;
        parent[b] = q;
        cl_next[keep_pos] = id;
    } else if (f & 1u) {
        cl_next[keep_pos] = cl[i];
    }
}

// The list's new length and the inner nodes made so far, from the last position's flags.
__global__ void k_ploc_state(const unsigned long long *__restrict__ flags,
                             const unsigned long long *__restrict__ excl, ploc_state *ps) {
    const int m = ps->m;
    if (m <= 1) return;
    const unsigned long long t = excl[m - 1] + flags[m - 1];
    ps->m = (int)(uint32_t)t;
    ps->made += (int)(t >> 32);
}

// Triangle counts of the inner nodes: creation order puts children before parents, so one
// pass per node in order would do; in parallel, each inner node climbs from its first-finished
// child with the second-arrival rule (an atomic per node; no thread waits for another).
__global__ void __launch_bounds__(kThreads) k_ploc_counts(const int2 *__restrict__ kid, const int32_t *__restrict__ parent,
                                                          int n, uint32_t *visits, int32_t *cnt, ploc_state *ps) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int q = parent[k];
    for (int climb = 0; climb < kMaxClimb && q >= 0; ++climb) {
        if (q >= n - 1) {
            atomicOr(&ps->err, 2);
            return;
        }
        __threadfence();
        if (atomicAdd(visits + q, 1u) == 0u) return;  // the sibling's thread continues
        __threadfence();
        const int2 c = kid[q];
        const int ca = c.x < n ? 1 : __ldcg(cnt + (c.x - n)), cb = c.y < n ? 1 : __ldcg(cnt + (c.y - n));
        cnt[q] = ca + cb;
        q = parent[n + q];
    }
    if (q >= 0) atomicOr(&ps->err, 4);
}

__device__ __forceinline__ int ploc_size(const int32_t *cnt, int n, int id) { return id < n ? 1 : cnt[id - n]; }

// Depth-first start position of every cluster id (its subtree's first triangle): the sizes of
// the left siblings of all its right-hand ancestors. Then the radix-tree form: inner node q
// becomes n - 2 - q (the root, made last, becomes 0), a triangle at sorted position k becomes
// leaf position pos(k), and `order2` lists the primitives in depth-first order.
__global__ void __launch_bounds__(kThreads) k_ploc_emit(const int2 *__restrict__ kid, const int32_t *__restrict__ parent,
                                                        const int32_t *__restrict__ cnt,
                                                        const uint32_t *__restrict__ order, int n, int2 *children,
                                                        int2 *range, int32_t *parent_inner, int32_t *parent_leaf,
                                                        uint32_t *order2, ploc_state *ps) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;  // cluster id: 0..n-1 triangles, n..2n-2 inner
    if (x >= 2 * n - 1) return;
    int start = 0, v = x, climb = 0;
    for (; climb < kMaxClimb && parent[v] >= 0; ++climb) {
        const int q = parent[v];
        if (q >= n - 1) {
            atomicOr(&ps->err, 8);
            return;
        }
        const int2 c = kid[q];
        if (c.y == v) start += ploc_size(cnt, n, c.x);
        v = n + q;
    }
    if (climb >= kMaxClimb || v != 2 * n - 2 || start < 0 || start >= n) {
        atomicOr(&ps->err, 16);
        return;
    }
    if (x < n) {
        order2[start] = order[x];
        const int p = parent[x];
        parent_leaf[start] = p >= 0 ? n - 2 - p : -1;
    } else {
        const int q = x - n, me = n - 2 - q;
        const int2 c = kid[q];
        range[me] = make_int2(start, start + cnt[q] - 1);
        const int p = parent[x];
        parent_inner[me] = p >= 0 ? n - 2 - p : -1;
        // children: inner nodes by their new numbers, triangles by their depth-first positions
        // (a triangle's position is its parent's start, plus the left sibling's size if right)
        const int l = c.x < n ? ~start : n - 2 - (c.x - n);
        const int r = c.y < n ? ~(start + ploc_size(cnt, n, c.x)) : n - 2 - (c.y - n);
        children[me] = make_int2(l, r);
    }
}

// What a child hands to its parent in the bottom-up pass (two per inner node).
struct slot {
    float4 lo;    // w: area-weighted cost S of the subtree
    float4 hi;    // w: triangle count (as float, exact below 2^24)
    int4 meta;    // x: child reference, y: height, z: 4-wide bound if inner else -1, w: M (see below)
};

__device__ __forceinline__ slot load_slot(const slot *p) {
    slot s;
    s.lo = __ldcg(&p->lo);
    s.hi = __ldcg(&p->hi);
    s.meta = __ldcg(&p->meta);
    return s;
}

// 4. bottom-up fit, SAH collapse and binary node output (`every_small_subtree`: every subtree of
// at most max_leaf triangles becomes a leaf, the reference's rule, for the SAH method's trees,
// which are split down to single triangles). For the 4-wide stack bound every inner
// node also carries B (the bound of a 4-wide node placed there: its wide children less one plus
// the largest B among its inner grandchildren) and M (the largest B among its inner children).
__global__ void __launch_bounds__(kThreads) k_bottom_up(const float4 *__restrict__ plo, const float4 *__restrict__ phi,
                                                        const uint32_t *__restrict__ order, int n, int max_leaf,
                                                        int every_small_subtree,
                                                        const int2 *__restrict__ children,
                                                        const int2 *__restrict__ range,
                                                        const int32_t *__restrict__ parent_inner,
                                                        const int32_t *__restrict__ parent_leaf, slot *slots,
                                                        uint32_t *visits, uint8_t *collapsed, float4 *nodes,
                                                        int32_t *info) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t prim = order[k];
    slot me;
    me.lo = plo[prim];
    me.hi = phi[prim];
    me.lo.w = half_area(me.lo, me.hi);
    me.hi.w = 1.f;
    me.meta = make_int4(~(k << 4), 0, -1, 0);
    if (n == 1) {
        info[GB_ROOT] = me.meta.x;
        info[GB_DEPTH] = 0;
        info[GB_ROOT4] = me.meta.x;
        info[GB_BOUND4] = 0;
        return;
    }
    int node = parent_leaf[k];
    if (node < 0 || node >= n - 1) {
        atomicOr(info + GB_ERR, GB_ERR_TREE);
        return;
    }
    bool left = children[node].x == ~k;
    for (int climb = 0; climb < kMaxClimb; ++climb) {
        slots[2 * node + (left ? 0 : 1)] = me;
        __threadfence();
        if (atomicAdd(visits + node, 1u) == 0u) return;  // the sibling's thread continues
        __threadfence();
        const slot a = load_slot(slots + 2 * node), b = load_slot(slots + 2 * node + 1);
        slot p;
        p.lo = make_float4(fminf(a.lo.x, b.lo.x), fminf(a.lo.y, b.lo.y), fminf(a.lo.z, b.lo.z), 0.f);
        p.hi = make_float4(fmaxf(a.hi.x, b.hi.x), fmaxf(a.hi.y, b.hi.y), fmaxf(a.hi.z, b.hi.z), 0.f);
        const float area = half_area(p.lo, p.hi);
        const float cnt = a.hi.w + b.hi.w;
        const float keep = area + a.lo.w + b.lo.w;
        const float as_leaf = area * cnt;
        const bool leaf = cnt <= (float)max_leaf && (every_small_subtree || !(as_leaf > keep));
        collapsed[node] = leaf ? 1 : 0;
        if (leaf) {
            p.lo.w = as_leaf;
            p.meta = make_int4(~((range[node].x << 4) | ((int)cnt - 1)), 0, -1, 0);
        } else {
            p.lo.w = keep;
            const bool ai = a.meta.z >= 0, bi = b.meta.z >= 0;
            const int wide_kids = (ai ? 2 : 1) + (bi ? 2 : 1);
            const int bnd = wide_kids - 1 + max(ai ? a.meta.w : 0, bi ? b.meta.w : 0);
            const int m = max(ai ? a.meta.z : 0, bi ? b.meta.z : 0);
            p.meta = make_int4(node, 1 + max(a.meta.y, b.meta.y), bnd, m);
            float4 *o = nodes + 4 * (size_t)node;
            o[0] = make_float4(a.lo.x, a.lo.y, a.hi.x, a.hi.y);
            o[1] = make_float4(a.lo.z, a.hi.z, __int_as_float(a.meta.x), 0.f);
            o[2] = make_float4(b.lo.x, b.lo.y, b.hi.x, b.hi.y);
            o[3] = make_float4(b.lo.z, b.hi.z, __int_as_float(b.meta.x), 0.f);
        }
        p.hi.w = cnt;
        if (node == 0) {
            info[GB_ROOT] = p.meta.x;
            info[GB_DEPTH] = p.meta.y;
            info[GB_ROOT4] = leaf ? p.meta.x : 0;
            info[GB_BOUND4] = leaf ? 0 : p.meta.z;
            return;
        }
        me = p;
        const int up = parent_inner[node];
        if (up < 0 || up >= n - 1) {
            atomicOr(info + GB_ERR, GB_ERR_TREE);
            return;
        }
        left = children[up].x == node;
        node = up;
    }
    atomicOr(info + GB_ERR, GB_ERR_DEPTH);
}

// ---- 4b. depth-first layout of the inner nodes ----------------------------------------------
//
// The radix tree numbers inner nodes by split position and PLOC by creation; neither keeps a
// node near the child a ray visits next. The host flattener keeps the reference's preorder (a
// parent followed by its left subtree, so the left child shares the parent's 128-byte line
// pair), and these passes give GPU-built trees the same layout: which inner nodes are in the
// final tree (no collapsed ancestor), the inner-node count of every subtree (bottom-up, second
// arrival continues), every node's preorder position (the sum, over its ancestors, of one plus
// the left sibling subtree's count where the path turns right), and the scatter of the nodes
// to their positions with their child references renumbered.

__device__ __forceinline__ int child_ref_of(const float4 *nodes, int i, int side) {
    return __float_as_int(nodes[4 * (size_t)i + 2 * side + 1].z);
}

__global__ void __launch_bounds__(kThreads) k_reach(int n, const uint8_t *__restrict__ collapsed,
                                                    const int32_t *__restrict__ parent_inner, int32_t *reach,
                                                    int32_t *info) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int r = 0;
    if (i < n - 1 && !collapsed[i]) {
        r = 1;
        int q = i, climb = 0;
        for (; q != 0 && climb < kMaxClimb; ++climb) {
            q = parent_inner[q];
            if (q < 0 || q >= n - 1) {
                atomicOr(info + GB_ERR, GB_ERR_TREE);
                r = 0;
                break;
            }
            if (collapsed[q]) {
                r = 0;
                break;
            }
        }
        if (climb >= kMaxClimb) {
            atomicOr(info + GB_ERR, GB_ERR_DEPTH);
            r = 0;
        }
    }
    reach[i] = r;
}

// Inner-node count of every final subtree; threads start at the final tree's bottom inner nodes.
__global__ void __launch_bounds__(kThreads) k_icount(int n, const float4 *__restrict__ nodes,
                                                     const int32_t *__restrict__ parent_inner,
                                                     const int32_t *__restrict__ reach, uint32_t *arrive,
                                                     int32_t *icount, int32_t *info) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1 || !reach[i]) return;
    if (child_ref_of(nodes, i, 0) >= 0 || child_ref_of(nodes, i, 1) >= 0) return;
    icount[i] = 1;
    int v = i;
    for (int climb = 0; climb < kMaxClimb; ++climb) {
        if (v == 0) return;
        const int p = parent_inner[v];
        if (p < 0 || p >= n - 1) {
            atomicOr(info + GB_ERR, GB_ERR_TREE);
            return;
        }
        const int l = child_ref_of(nodes, p, 0), r = child_ref_of(nodes, p, 1);
        if (l >= n - 1 || r >= n - 1) {
            atomicOr(info + GB_ERR, GB_ERR_TREE);
            return;
        }
        __threadfence();
        if (l >= 0 && r >= 0 && atomicAdd(arrive + p, 1u) == 0u) return;  // the sibling's thread continues
        __threadfence();
        icount[p] = 1 + (l >= 0 ? __ldcg(icount + l) : 0) + (r >= 0 ? __ldcg(icount + r) : 0);
        v = p;
    }
    atomicOr(info + GB_ERR, GB_ERR_DEPTH);
}

__global__ void __launch_bounds__(kThreads) k_dfs_pos(int n, const float4 *__restrict__ nodes,
                                                      const int32_t *__restrict__ parent_inner,
                                                      const int32_t *__restrict__ reach,
                                                      const int32_t *__restrict__ icount, int32_t *pos,
                                                      int32_t *info) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1 || !reach[i]) return;
    int s = 0, v = i, climb = 0;
    for (; v != 0 && climb < kMaxClimb; ++climb) {
        const int p = parent_inner[v];
        if (p < 0 || p >= n - 1) {
            atomicOr(info + GB_ERR, GB_ERR_TREE);
            return;
        }
        const int l = child_ref_of(nodes, p, 0);
        s += 1 + ((l >= 0 && l != v) ? icount[l] : 0);
        v = p;
    }
    if (v != 0 || s >= n - 1) {
        atomicOr(info + GB_ERR, GB_ERR_TREE);
        return;
    }
    pos[i] = s;
}

// The final tree's inner nodes at their preorder positions, inner child references renumbered;
// parents and collapse flags in the new numbering (positions beyond the tree stay collapsed).
__global__ void __launch_bounds__(kThreads) k_relayout(int n, const float4 *__restrict__ nodes,
                                                       const int32_t *__restrict__ parent_inner,
                                                       const int32_t *__restrict__ reach,
                                                       const int32_t *__restrict__ pos, float4 *out_nodes,
                                                       int32_t *out_parent, uint8_t *out_collapsed) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1 || !reach[i]) return;
    const int j = pos[i];
    if (j < 0 || j >= n - 1) return;
    const float4 *src = nodes + 4 * (size_t)i;
    float4 *dst = out_nodes + 4 * (size_t)j;
    for (int side = 0; side < 2; ++side) {
        float4 xy = src[2 * side], z = src[2 * side + 1];
        const int c = __float_as_int(z.z);
        if (c >= 0 && c < n - 1) z.z = __int_as_float(pos[c]);
        dst[2 * side] = xy;
        dst[2 * side + 1] = z;
    }
    out_parent[j] = i == 0 ? -1 : pos[parent_inner[i]];
    out_collapsed[j] = 0;
}

// records in sorted order: v0 + original id, v0 - v1 + material, v0 - v2
__global__ void __launch_bounds__(kThreads) k_records(const float4 *__restrict__ vpos, const uint4 *__restrict__ tris,
                                                      const uint32_t *__restrict__ order, uint32_t n, uint32_t nv,
                                                      float4 *records) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t prim = order[k];
    const uint4 t = tris[prim];
    float4 a = make_float4(0.f, 0.f, 0.f, 0.f), b = a, c = a;
    if (t.x < nv && t.y < nv && t.z < nv) {
        a = vpos[t.x];
        b = vpos[t.y];
        c = vpos[t.z];
    }
    float4 *r = records + 3 * (size_t)k;
    r[0] = make_float4(a.x, a.y, a.z, __uint_as_float(prim));
    r[1] = make_float4(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z), __uint_as_float(t.w));
    r[2] = make_float4(__fsub_rn(a.x, c.x), __fsub_rn(a.y, c.y), __fsub_rn(a.z, c.z), 0.f);
}

// 5a. which inner nodes become 4-wide nodes: reachable (no collapsed ancestor) and at even depth
__global__ void __launch_bounds__(kThreads) k_wide_flags(int n, const uint8_t *__restrict__ collapsed,
                                                         const int32_t *__restrict__ parent_inner,
                                                         const float4 *__restrict__ nodes, int32_t *flag,
                                                         int32_t *links, int32_t *info) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int f = 0;
    if (i < n - 1 && !collapsed[i]) {
        int depth = 0, q = i;
        bool reach = true;
        while (q != 0 && depth < kMaxClimb) {
            q = parent_inner[q];
            ++depth;
            if (q < 0 || q >= n - 1) {
                atomicOr(info + GB_ERR, GB_ERR_TREE);
                reach = false;
                break;
            }
            if (collapsed[q]) {
                reach = false;
                break;
            }
        }
        if (depth >= kMaxClimb) {
            atomicOr(info + GB_ERR, GB_ERR_DEPTH);
            reach = false;
        }
        if (reach) {
            atomicAdd(info + GB_INNER, 1);
            f = (depth & 1) == 0;
            if (links) {  // refit links of the node's inner children: (parent << 1) | side
                const int cl = __float_as_int(nodes[4 * (size_t)i + 1].z), cr = __float_as_int(nodes[4 * (size_t)i + 3].z);
                if (cl >= 0 && cl < n - 1) links[cl] = 2 * i;
                if (cr >= 0 && cr < n - 1) links[cr] = 2 * i + 1;
            }
        }
    }
    flag[i] = f;
}

// 5b. wide index of every flagged node (exclusive sum of the flags, -1 elsewhere) and the count
__global__ void __launch_bounds__(kThreads) k_wide_index(int n, const int32_t *__restrict__ flag,
                                                         const int32_t *__restrict__ excl, int32_t *wide_index,
                                                         int32_t *info) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    wide_index[i] = flag[i] ? excl[i] : -1;
    if (i == n - 1) info[GB_WIDE_NODES] = excl[i] + flag[i];
}

// 5c. the 4-wide nodes (four child records, unused slots +inf / kEmptyWideChild)
__global__ void __launch_bounds__(kThreads) k_wide_nodes(const float4 *__restrict__ nodes,
                                                         const int32_t *__restrict__ wide_index, int n,
                                                         float4 *nodes4) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const int w = wide_index[p];
    if (w < 0) return;
    float lo[3][4], hi[3][4];
    int ref[4];
    int k = 0;
    const float4 *np = nodes + 4 * (size_t)p;
    for (int side = 0; side < 2; ++side) {
        const float4 bxy = np[2 * side], bz = np[2 * side + 1];  // (lo.x, lo.y, hi.x, hi.y), (lo.z, hi.z, ref, 0)
        const int c = __float_as_int(bz.z);
        if (c >= n - 1) return;  // not a node of this tree (never for a tree of k_bottom_up)
        if (c >= 0) {
            const float4 *cp = nodes + 4 * (size_t)c;
            for (int g = 0; g < 2; ++g) {
                const float4 gxy = cp[2 * g], gz = cp[2 * g + 1];
                const int gc = __float_as_int(gz.z);
                if (gc >= n - 1) return;
                lo[0][k] = gxy.x, lo[1][k] = gxy.y, lo[2][k] = gz.x;
                hi[0][k] = gxy.z, hi[1][k] = gxy.w, hi[2][k] = gz.y;
                ref[k++] = gc >= 0 ? wide_index[gc] : gc;
            }
        } else {
            lo[0][k] = bxy.x, lo[1][k] = bxy.y, lo[2][k] = bz.x;
            hi[0][k] = bxy.z, hi[1][k] = bxy.w, hi[2][k] = bz.y;
            ref[k++] = c;
        }
    }
    const float inf = __int_as_float(0x7f800000);
    for (; k < 4; ++k) {
        for (int a = 0; a < 3; ++a) lo[a][k] = hi[a][k] = inf;
        ref[k] = kEmptyWideChild;
    }
    float4 *o = nodes4 + 8 * (size_t)w;
    for (int i = 0; i < 4; ++i) {  // child records as in the binary layout
        o[2 * i] = make_float4(lo[0][i], lo[1][i], hi[0][i], hi[1][i]);
        o[2 * i + 1] = make_float4(lo[2][i], hi[2][i], __int_as_float(ref[i]), 0.f);
    }
}

// bounds: centre min (3), centre max (3), box min (3), box max (3), ordered-encoded
__global__ void k_init_info(int32_t *info, uint32_t *cbounds) {
    if (threadIdx.x < 8) info[threadIdx.x] = threadIdx.x == GB_FINITE ? 1 : 0;
    const unsigned t = threadIdx.x;
    if (t < 12) cbounds[t] = bound_is_min(t) ? 0xffffffffu : 0u;
}

inline size_t up256(size_t b) { return (b + 255) & ~(size_t)255; }

// scratch layout for up to n triangles (the PLOC arrays only when `ploc`)
struct arena {
    float4 *lo, *hi;
    uint32_t *keys_a, *keys_b, *vals_a, *vals_b, *cbounds, *visits;
    int2 *children, *range;
    int32_t *parent_inner, *parent_leaf, *flag, *excl;
    slot *slots;
    uint8_t *collapsed;
    // PLOC: cluster lists, boxes and parents of all 2n - 1 cluster ids, children of the inner
    // nodes made, nearest neighbours, merge flags and their prefix sums, subtree sizes, the
    // depth-first primitive order, the climbing counters and the iteration state
    int32_t *cl_a, *cl_b, *pparent, *nn, *cnt;
    float4 *box_lo, *box_hi;
    int2 *kid;
    unsigned long long *pflags, *pexcl;
    uint32_t *order2, *pvisits;
    ploc_state *ps;
    void *sah;  // the SAH method's scratch (gpu_build_sah.cu)
    void *cub;
    size_t cub_bytes, total;
};

size_t cub_bytes_for(uint32_t n) {
    size_t a = 0, b = 0, c = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, a, (const uint32_t *)nullptr, (uint32_t *)nullptr,
                                    (const uint32_t *)nullptr, (uint32_t *)nullptr, (int)n, 0, 30);
    cub::DeviceScan::ExclusiveSum(nullptr, b, (const int32_t *)nullptr, (int32_t *)nullptr, (int)n);
    cub::DeviceScan::ExclusiveSum(nullptr, c, (const unsigned long long *)nullptr, (unsigned long long *)nullptr,
                                  (int)n);
    return std::max(a, std::max(b, c));
}

arena carve(void *base, uint32_t n, int method) {
    const bool ploc = method == GB_METHOD_PLOC;
    arena A{};
    char *p = (char *)base;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        void *r = p ? p + off : nullptr;
        off += up256(bytes);
        return r;
    };
    const size_t m = n > 0 ? n : 1;
    A.lo = (float4 *)take(m * 16);
    A.hi = (float4 *)take(m * 16);
    A.keys_a = (uint32_t *)take(m * 4);
    A.keys_b = (uint32_t *)take(m * 4);
    A.vals_a = (uint32_t *)take(m * 4);
    A.vals_b = (uint32_t *)take(m * 4);
    A.cbounds = (uint32_t *)take(16 * 4);
    A.visits = (uint32_t *)take(m * 4);
    A.children = (int2 *)take(m * 8);
    A.range = (int2 *)take(m * 8);
    A.parent_inner = (int32_t *)take(m * 4);
    A.parent_leaf = (int32_t *)take(m * 4);
    A.flag = (int32_t *)take(m * 4);
    A.excl = (int32_t *)take(m * 4);
    A.slots = (slot *)take(m * 2 * sizeof(slot));
    A.collapsed = (uint8_t *)take(m);
    if (ploc) {
        A.cl_a = (int32_t *)take(m * 4);
        A.cl_b = (int32_t *)take(m * 4);
        A.pparent = (int32_t *)take(2 * m * 4);
        A.nn = (int32_t *)take(m * 4);
        A.cnt = (int32_t *)take(m * 4);
        A.box_lo = (float4 *)take(2 * m * 16);
        A.box_hi = (float4 *)take(2 * m * 16);
        A.kid = (int2 *)take(m * 8);
        A.pflags = (unsigned long long *)take(m * 8);
        A.pexcl = (unsigned long long *)take(m * 8);
        A.order2 = (uint32_t *)take(m * 4);
        A.pvisits = (uint32_t *)take(m * 4);
        A.ps = (ploc_state *)take(sizeof(ploc_state));
    }
    if (method == GB_METHOD_SAH) A.sah = take(sah_scratch_bytes((uint32_t)m));
    A.cub_bytes = cub_bytes_for((uint32_t)m);
    A.cub = take(A.cub_bytes);
    A.total = off;
    return A;
}

inline unsigned blocks_for(uint32_t n) { return (n + kThreads - 1) / kThreads; }

}  // namespace

namespace {
struct pinned_word {
    int32_t *p = nullptr;
    int32_t fallback = 0;
    pinned_word() {
        if (cudaMallocHost((void **)&p, sizeof(int32_t)) != cudaSuccess) {
            cudaGetLastError();
            p = nullptr;
        }
    }
    ~pinned_word() {
        if (p) cudaFreeHost(p);
    }
};
}  // namespace

int32_t *readback_word() {
    thread_local pinned_word w;
    return w.p ? w.p : &w.fallback;
}

size_t gpu_build_scratch_bytes(uint32_t max_tris, int method) {
    return carve(nullptr, max_tris, method).total;
}

namespace {

__global__ void k_ploc_report(const ploc_state *ps, int32_t *info) {
    if (ps->err || ps->m != 1) atomicOr(info + GB_ERR, GB_ERR_TREE);
}

// Iterations of nearest-neighbour merging before the remaining clusters are paired by position,
// and the number of pairing iterations that always finishes the tree.
int ploc_budget(uint32_t n) {
    int lg = 0;
    while ((1u << lg) < n) ++lg;
    return 48 + 2 * lg;
}
int ploc_pairing_rounds(uint32_t n) {
    int lg = 0;
    while ((1u << lg) < n) ++lg;
    return lg + 1;
}

// The PLOC tree of the n >= 2 sorted triangles in the radix tree's form (children, range,
// parent_inner, parent_leaf) with its depth-first primitive order in A.order2. The list length
// is read back every 8 iterations, so that no launch is made once the tree is finished.
cudaError_t ploc_tree(const arena &A, int n, cudaStream_t st) {
    const unsigned nb = (n + kThreads - 1) / kThreads;
    k_ploc_init<<<nb, kThreads, 0, st>>>(A.lo, A.hi, A.vals_b, n, A.cl_a, A.box_lo, A.box_hi, A.pparent, A.ps);
    int32_t *cur = A.cl_a, *next = A.cl_b;
    const int budget = ploc_budget((uint32_t)n), total = budget + ploc_pairing_rounds((uint32_t)n);
    cudaError_t e = cudaGetLastError();
    for (int it = 0; it < total && e == cudaSuccess; ++it) {
        if (it % 8 == 7) {  // stop once one cluster is left
            int32_t *m = readback_word();
            e = cudaMemcpyAsync(m, &A.ps->m, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            if (e != cudaSuccess || *m <= 1) break;
        }
        k_ploc_nn<<<nb, kThreads, 0, st>>>(cur, A.box_lo, A.box_hi, A.ps, it >= budget ? 1 : 0, A.nn);
        k_ploc_flags<<<nb, kThreads, 0, st>>>(A.nn, A.ps, n, A.pflags);
        size_t cb = A.cub_bytes;
        e = cub::DeviceScan::ExclusiveSum(A.cub, cb, A.pflags, A.pexcl, n, st);
        if (e != cudaSuccess) break;
        k_ploc_apply<<<nb, kThreads, 0, st>>>(cur, A.nn, A.pflags, A.pexcl, n, A.ps, A.kid, A.box_lo, A.box_hi,
                                              A.pparent, next);
        k_ploc_state<<<1, 1, 0, st>>>(A.pflags, A.pexcl, A.ps);
        std::swap(cur, next);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(A.pvisits, 0, (size_t)n * 4, st);
    if (e != cudaSuccess) return e;
    k_ploc_counts<<<nb, kThreads, 0, st>>>(A.kid, A.pparent, n, A.pvisits, A.cnt, A.ps);
    k_ploc_emit<<<(2 * n - 1 + kThreads - 1) / kThreads, kThreads, 0, st>>>(A.kid, A.pparent, A.cnt, A.vals_b, n,
                                                                         A.children, A.range, A.parent_inner,
                                                                         A.parent_leaf, A.order2, A.ps);
    return cudaGetLastError();
}

// The passes after the tree, for every method: boxes and leaf collapse bottom-up, the
// depth-first layout, the triangle records and the 4-wide indices. `A` holds the boxes and the
// tree (children, range, parent links) and the scratch; its visit counts are zero and its
// collapse flags one on entry.
cudaError_t build_tail(const arena &A, const float4 *vpos, uint32_t nv, const uint4 *tris, uint32_t nt, int max_leaf,
                       bool sah, const uint32_t *order, float4 *nodes, float4 *records, int32_t *wide_index,
                       int32_t *links, int32_t *info, cudaStream_t st) {
    const unsigned nb = blocks_for(nt);
    size_t cb = A.cub_bytes;
    cudaError_t e = cudaSuccess;
    k_bottom_up<<<nb, kThreads, 0, st>>>(A.lo, A.hi, order, (int)nt, max_leaf, sah ? 1 : 0, A.children, A.range,
                                         A.parent_inner, A.parent_leaf, A.slots, A.visits, A.collapsed, nodes,
                                         info);
    if (nt > 1) {
        // depth-first layout; the bottom-up pass's slots and the sort's key and value arrays are
        // free now and hold the new nodes, positions, parents and flags
        float4 *tmp_nodes = (float4 *)A.slots;
        int32_t *reach = A.flag, *icount = A.excl, *pos = (int32_t *)A.keys_a, *new_parent = (int32_t *)A.vals_a;
        uint8_t *new_collapsed = (uint8_t *)A.keys_b;
        e = cudaMemsetAsync(A.visits, 0, (size_t)nt * 4, st);
        if (e == cudaSuccess) e = cudaMemsetAsync(new_collapsed, 1, (size_t)nt, st);
        if (e == cudaSuccess) e = cudaMemsetAsync(new_parent, 0xff, (size_t)nt * 4, st);
        if (e != cudaSuccess) return e;
        k_reach<<<nb, kThreads, 0, st>>>((int)nt, A.collapsed, A.parent_inner, reach, info);
        k_icount<<<nb, kThreads, 0, st>>>((int)nt, nodes, A.parent_inner, reach, A.visits, icount, info);
        k_dfs_pos<<<nb, kThreads, 0, st>>>((int)nt, nodes, A.parent_inner, reach, icount, pos, info);
        k_relayout<<<nb, kThreads, 0, st>>>((int)nt, nodes, A.parent_inner, reach, pos, tmp_nodes, new_parent,
                                            new_collapsed);
        e = cudaMemcpyAsync(nodes, tmp_nodes, (size_t)(nt - 1) * 64, cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(A.parent_inner, new_parent, (size_t)nt * 4, cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(A.collapsed, new_collapsed, (size_t)nt, cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) return e;
    }
    k_records<<<nb, kThreads, 0, st>>>(vpos, tris, order, nt, nv, records);
    if (nt > 1) {
        k_wide_flags<<<nb, kThreads, 0, st>>>((int)nt, A.collapsed, A.parent_inner, nodes, A.flag, links, info);
        cb = A.cub_bytes;
        e = cub::DeviceScan::ExclusiveSum(A.cub, cb, A.flag, A.excl, (int)nt, st);
        if (e != cudaSuccess) return e;
        k_wide_index<<<nb, kThreads, 0, st>>>((int)nt, A.flag, A.excl, wide_index, info);
    }
    return cudaGetLastError();
}

}  // namespace

cudaError_t gpu_build_binary(const float4 *vpos, uint32_t nv, const uint4 *tris, uint32_t nt, int max_leaf,
                             void *scratch, size_t scratch_bytes, float4 *nodes, float4 *records,
                             int32_t *wide_index, int32_t *links, int32_t *info, int method, int planes,
                             cudaStream_t st) {
    const bool ploc = method == GB_METHOD_PLOC && nt > 1, sah = method == GB_METHOD_SAH && nt > 1;
    if (method == GB_METHOD_SAH && (planes < 1 || planes > kMaxSahPlanes)) return cudaErrorInvalidValue;
    arena A = carve(scratch, nt, method);
    if (A.total > scratch_bytes) return cudaErrorInvalidValue;
    k_init_info<<<1, 32, 0, st>>>(info, A.cbounds);
    if (nt == 0) return cudaGetLastError();
    const unsigned nb = blocks_for(nt);
    k_prims<<<nb, kThreads, 0, st>>>(vpos, nv, tris, nt, A.lo, A.hi, A.cbounds, info);
    size_t cb = A.cub_bytes;
    cudaError_t e = cudaSuccess;
    if (!sah) {
        k_morton<<<nb, kThreads, 0, st>>>(A.lo, A.hi, nt, A.cbounds, A.keys_a, A.vals_a);
        e = cub::DeviceRadixSort::SortPairs(A.cub, cb, A.keys_a, A.keys_b, A.vals_a, A.vals_b, (int)nt, 0, 30, st);
        if (e != cudaSuccess) return e;
    }
    // parents start at -1, so a position the tree misses is caught instead of read as an index
    e = cudaMemsetAsync(A.visits, 0, (size_t)nt * 4, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(A.collapsed, 1, (size_t)nt, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(A.parent_inner, 0xff, (size_t)nt * 4, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(A.parent_leaf, 0xff, (size_t)nt * 4, st);
    if (e == cudaSuccess && links) e = cudaMemsetAsync(links, 0xff, (size_t)nt * 4, st);
    if (e != cudaSuccess) return e;
    const uint32_t *order = A.vals_b;  // primitives in leaf order
    if (sah) {
        e = sah_tree(A.sah, nt, planes, A.lo, A.hi, A.cbounds + 6, A.children, A.range, A.parent_inner,
                     A.parent_leaf, A.flag, A.excl, A.cub, A.cub_bytes, &order, info, st);
        if (e != cudaSuccess) return e;
    } else if (ploc) {
        e = ploc_tree(A, (int)nt, st);
        if (e != cudaSuccess) return e;
        k_ploc_report<<<1, 1, 0, st>>>(A.ps, info);
        order = A.order2;
    } else if (nt > 1) {
        k_radix_tree<<<blocks_for(nt - 1), kThreads, 0, st>>>(A.keys_b, (int)nt, A.children, A.range,
                                                              A.parent_inner, A.parent_leaf);
    }
    return build_tail(A, vpos, nv, tris, nt, max_leaf, sah, order, nodes, records, wide_index, links, info, st);
}

sah_set sah_set_carve(void *base, uint32_t n_total, uint32_t count) {
    sah_set S{};
    char *p = (char *)base;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        void *r = p ? p + off : nullptr;
        off += up256(bytes);
        return r;
    };
    const size_t m = n_total > 0 ? n_total : 1, c = count > 0 ? count : 1;
    S.lo = (float4 *)take(m * 16);
    S.hi = (float4 *)take(m * 16);
    S.cbounds = (uint32_t *)take(c * 16 * 4);
    S.children = (int2 *)take(m * 8);
    S.range = (int2 *)take(m * 8);
    S.parent_inner = (int32_t *)take(m * 4);
    S.parent_leaf = (int32_t *)take(m * 4);
    S.flag = (int32_t *)take(m * 4);
    S.excl = (int32_t *)take(m * 4);
    S.scenes = (sah_set_scene *)take(c * sizeof(sah_set_scene));
    S.sah = take(sah_scratch_bytes((uint32_t)m));
    S.cub_bytes = cub_bytes_for((uint32_t)m);
    S.cub = take(S.cub_bytes);
    S.total = off;
    S.n = n_total;
    S.count = count;
    return S;
}

cudaError_t sah_set_prims(const sah_set &S, uint32_t i, uint32_t first, const float4 *vpos, uint32_t nv,
                          const uint4 *tris, uint32_t nt, int32_t *info, cudaStream_t st) {
    if (i >= S.count || (uint64_t)first + nt > S.n) return cudaErrorInvalidValue;
    uint32_t *cb = S.cbounds + 16 * (size_t)i;
    k_init_info<<<1, 32, 0, st>>>(info, cb);
    if (nt) k_prims<<<blocks_for(nt), kThreads, 0, st>>>(vpos, nv, tris, nt, S.lo + first, S.hi + first, cb, info);
    return cudaGetLastError();
}

cudaError_t sah_set_trees(const sah_set &S, const sah_set_scene *scenes_host, int planes, const uint32_t **order,
                          int32_t *set_info, cudaStream_t st) {
    if (S.n < 2 || S.count == 0 || planes < 1 || planes > kMaxSahPlanes) return cudaErrorInvalidValue;
    uint64_t at = 0;  // the scenes tile the positions in order
    for (uint32_t i = 0; i < S.count; ++i) {
        if (scenes_host[i].first != at) return cudaErrorInvalidValue;
        at += scenes_host[i].n;
    }
    if (at != S.n) return cudaErrorInvalidValue;
    cudaError_t e =
        cudaMemcpyAsync(S.scenes, scenes_host, S.count * sizeof(sah_set_scene), cudaMemcpyHostToDevice, st);
    // parents start at -1, so a position the tree misses is caught instead of read as an index
    if (e == cudaSuccess) e = cudaMemsetAsync(S.parent_inner, 0xff, (size_t)S.n * 4, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(S.parent_leaf, 0xff, (size_t)S.n * 4, st);
    if (e != cudaSuccess) return e;
    return sah_tree_set(S.sah, S.n, S.scenes, S.count, planes, S.lo, S.hi, S.cbounds, S.children, S.range,
                        S.parent_inner, S.parent_leaf, S.flag, S.excl, S.cub, S.cub_bytes, order, set_info, st);
}

cudaError_t sah_set_finish(const sah_set &S, const uint32_t *order, uint32_t first, const float4 *vpos,
                           uint32_t nv, const uint4 *tris, uint32_t nt, int max_leaf, void *scratch,
                           size_t scratch_bytes, float4 *nodes, float4 *records, int32_t *wide_index, int32_t *info,
                           cudaStream_t st) {
    if ((uint64_t)first + nt > S.n) return cudaErrorInvalidValue;
    arena A = carve(scratch, nt, GB_METHOD_LBVH);
    if (A.total > scratch_bytes) return cudaErrorInvalidValue;
    if (nt == 0) return cudaSuccess;
    // the boxes and the tree are the scene's slices of the set's arrays, the rest is `scratch`
    A.lo = S.lo + first;
    A.hi = S.hi + first;
    A.children = S.children + first;
    A.range = S.range + first;
    A.parent_inner = S.parent_inner + first;
    A.parent_leaf = S.parent_leaf + first;
    cudaError_t e = cudaMemsetAsync(A.visits, 0, (size_t)nt * 4, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(A.collapsed, 1, (size_t)nt, st);
    if (e != cudaSuccess) return e;
    return build_tail(A, vpos, nv, tris, nt, max_leaf, nt > 1, order + first, nodes, records, wide_index, nullptr,
                      info, st);
}

cudaError_t gpu_build_wide(const float4 *nodes, const int32_t *wide_index, uint32_t nt, float4 *nodes4,
                           cudaStream_t st) {
    if (nt < 2) return cudaSuccess;
    k_wide_nodes<<<blocks_for(nt), kThreads, 0, st>>>(nodes, wide_index, (int)nt, nodes4);
    return cudaGetLastError();
}

}  // namespace grt
