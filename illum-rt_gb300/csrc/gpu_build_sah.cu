// Top-down SAH construction on the GPU with the reference's split rule (rt/cpu/bvh-ctor.h:386-488):
// a node is split on the major axis of its box at one of `planes` evenly spaced candidate planes
// (as many as it has primitives when that is fewer), primitives whose box centre lies at or below
// the plane going left; the candidate of least (A_l / A) n_l + (A_r / A) n_r wins, the first one
// on ties; when a plane leaves one side empty, the split at the median of the centres is a
// candidate in its place (once). Where the reference partitions and sorts primitives in place,
// this builder bins them, so its trees differ from the reference's in detail (not in quality):
// the reference's in-place partition never classifies the element where its two pointers meet,
// this one classifies every primitive, and equal centres are ordered by position; and for nodes
// of more than kSmall primitives, whose planes are closely spaced, the median (taken there in
// position order) is used only when no plane separates the node.
//
// The output is a full binary tree over single primitives in the form the bottom-up pass of
// gpu_build.cu takes (children, range, parent links, the primitive order), whose leaf collapse
// then makes every subtree of at most max_tris primitives a leaf, as the reference's
// subdivision stops there (rt/cpu/bvh-ctor.h:371-380).
//
// Inner nodes are numbered in preorder without any counter: a node of m primitives owns the
// m - 1 numbers from its own, its left child (n_l primitives) takes the next one and its right
// child the number n_l after its own, so the numbering and every result are independent of
// thread timing.
//
// Two phases:
//   * large nodes (more than kSmall primitives), one level of the tree per round: every
//     primitive's centre binned into its node's candidate intervals (global atomics into a bin
//     array that gives node k of the level the slots from first_k + k), one warp per node
//     scanning its bins for the best plane, a stable partition (a device-wide prefix sum of
//     the left flags), and the children of the level listed in position order for the next
//     round (a second prefix sum), small ones set aside;
//   * small nodes, one warp each: the primitives in shared memory, the whole subtree built with
//     an explicit stack, every candidate plane evaluated by its own lane.
#include <cub/device/device_scan.cuh>

#include <cfloat>
#include <climits>

#include "gpu_build.hpp"
#include "grt_internal.hpp"

namespace grt {
namespace {

constexpr int kT = 256;
constexpr int kSmall = 32;     // nodes of at most this many primitives: one warp builds the subtree
constexpr int kChooseWarps = 4;
constexpr int kSmallWarps = 4;
constexpr unsigned kFull = 0xffffffffu;

// A node still to split: its box, its number, and the positions [first, end) of its primitives.
struct sah_task {
    float4 lo, hi;  // w unused
    int4 m;         // (node number, first, end, 0)
};
// The split chosen for a large node: child boxes, and (median?, plane, n_left).
struct sah_split {
    float4 llo, lhi, rlo, rhi;
    int4 m;
};
// One candidate interval of a large node: primitive count and the box of their boxes, the
// bounds in the order-preserving unsigned encoding (so that atomicMin / atomicMax order them).
struct sah_bin {
    uint32_t cnt, lo[3], hi[3], pad;
};

__device__ __forceinline__ uint32_t ordered(float f) {
    const uint32_t b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float unordered(uint32_t u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

__device__ __forceinline__ float comp(const float4 &v, int a) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); }

// bvh-ctor.h:387-390, every operation rounded as written
__device__ __forceinline__ float surface_rn(float lx, float ly, float lz, float hx, float hy, float hz) {
    const float ex = __fsub_rn(hx, lx), ey = __fsub_rn(hy, ly), ez = __fsub_rn(hz, lz);
    return __fmul_rn(2.f, __fadd_rn(__fadd_rn(__fmul_rn(ex, ey), __fmul_rn(ex, ez)), __fmul_rn(ey, ez)));
}
// the largest extent with the tie order x, y, z (bvh-ctor.h:397-398)
__device__ __forceinline__ int major_axis(float lx, float ly, float lz, float hx, float hy, float hz) {
    const float ex = __fsub_rn(hx, lx), ey = __fsub_rn(hy, ly), ez = __fsub_rn(hz, lz);
    float m = (ey < ez) ? ez : ey;
    m = (ex < m) ? m : ex;
    return m == ex ? 0 : (m == ey ? 1 : 2);
}
__device__ __forceinline__ float centre(float lo, float hi) { return __fmul_rn(__fadd_rn(lo, hi), 0.5f); }

// candidate plane i of P on [lo, lo + ext]: lo + (i + 1) (ext / (P + 1)) (bvh-ctor.h:415)
__device__ __forceinline__ float plane_at(float lo, float q, int i) { return __fadd_rn(lo, __fmul_rn((float)(i + 1), q)); }

// The interval of centre c: the first plane i with c <= plane i, P when there is none (also for
// a NaN centre). Planes grow with i, so the estimate is corrected by stepping.
__device__ __forceinline__ int bin_of(float c, float lo, float q, int P) {
    if (c != c) return P;
    float g = __fdiv_rn(__fsub_rn(c, lo), q) - 1.f;
    g = fminf(fmaxf(g, 0.f), (float)P);  // also maps a NaN estimate to 0
    int i = (int)g;
    while (i > 0 && c <= plane_at(lo, q, i - 1)) --i;
    while (i < P && !(c <= plane_at(lo, q, i))) ++i;
    return i;
}

__global__ void k_iota(uint32_t *v, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v[i] = i;
}

__global__ void k_sah_clear(sah_bin *bins, size_t n) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    bins[i] = sah_bin{0u, {kFull, kFull, kFull}, {0u, 0u, 0u}, 0u};
}

// The root: the box of all primitive boxes (ordered bounds from the primitive pass) and every
// position; into the large list, or the small one for a scene of at most kSmall triangles.
__global__ void k_sah_root(const uint32_t *bounds, int n, sah_task *large, int *n_large, sah_task *small,
                           int *n_small) {
    if (threadIdx.x != 0) return;
    sah_task t;
    t.lo = make_float4(unordered(bounds[0]), unordered(bounds[1]), unordered(bounds[2]), 0.f);
    t.hi = make_float4(unordered(bounds[3]), unordered(bounds[4]), unordered(bounds[5]), 0.f);
    t.m = make_int4(0, 0, n, 0);
    if (n > kSmall) {
        large[0] = t;
        *n_large = 1;
        *n_small = 0;
    } else {
        small[0] = t;
        *n_large = 0;
        *n_small = 1;
    }
}

// The roots of a scene set (one warp): the scenes of more than kSmall primitives into the large
// list in scene order, so that the list is sorted by first position like every later level's,
// the scenes of 2 .. kSmall primitives into the small list. Scene i's primitives are the
// positions [first, first + n) and its inner nodes are numbered from first.
__global__ void k_sah_roots(const sah_set_scene *__restrict__ scenes, int count, const uint32_t *__restrict__ cbounds,
                            sah_task *large, int *n_large, sah_task *small, int *n_small) {
    const int lane = threadIdx.x & 31;
    if (threadIdx.x >= 32) return;
    const unsigned below = (1u << lane) - 1u;
    int nlarge = 0, nsmall = 0;
    for (int c0 = 0; c0 < count; c0 += 32) {
        const int i = c0 + lane;
        sah_task t{};
        int n = 0;
        if (i < count) {
            const sah_set_scene sc = scenes[i];
            const uint32_t *b = cbounds + 16 * (size_t)i + 6;  // the box bounds of the primitive pass
            n = (int)sc.n;
            t.lo = make_float4(unordered(b[0]), unordered(b[1]), unordered(b[2]), 0.f);
            t.hi = make_float4(unordered(b[3]), unordered(b[4]), unordered(b[5]), 0.f);
            t.m = make_int4((int)sc.first, (int)sc.first, (int)(sc.first + sc.n), 0);
        }
        const bool is_large = n > kSmall, is_small = n >= 2 && n <= kSmall;
        const unsigned lm = __ballot_sync(kFull, is_large), sm = __ballot_sync(kFull, is_small);
        if (is_large) large[nlarge + __popc(lm & below)] = t;
        if (is_small) small[nsmall + __popc(sm & below)] = t;
        nlarge += __popc(lm);
        nsmall += __popc(sm);
    }
    if (lane == 0) {
        *n_large = nlarge;
        *n_small = nsmall;
    }
}

// Scene i of a set whose position j lies in [first, first + n): the last scene whose first
// position is at most j (an empty scene shares its first position with the scene after it).
__device__ __forceinline__ int scene_of_pos(const sah_set_scene *scenes, int count, uint32_t j) {
    int lo = 0, hi = count - 1, k = 0;
    while (lo <= hi) {
        const int mid = (lo + hi) >> 1;
        if (scenes[mid].first <= j) {
            k = mid;
            lo = mid + 1;
        } else {
            hi = mid - 1;
        }
    }
    return k;
}

// A scene set's tree arrays in every scene's own numbering: positions, inner nodes and
// primitives of scene i less its first position (leaf references are complemented positions).
// Slot first + n - 1 of a scene holds no inner node; converting what it holds does no harm.
__global__ void __launch_bounds__(kT) k_sah_localize(const sah_set_scene *__restrict__ scenes, int count, int n,
                                                     int2 *children, int2 *range, int32_t *parent_inner,
                                                     int32_t *parent_leaf, uint32_t *order) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const uint32_t f = scenes[scene_of_pos(scenes, count, (uint32_t)j)].first;
    // in unsigned arithmetic, so that an unused slot's contents cannot overflow
    auto less = [f](int v) { return (int)((uint32_t)v - f); };
    auto ref = [f](int v) { return v >= 0 ? (int)((uint32_t)v - f) : (int)~((uint32_t)~v - f); };
    order[j] -= f;
    const int pl = parent_leaf[j];
    if (pl >= 0) parent_leaf[j] = less(pl);
    const int pi = parent_inner[j];
    if (pi >= 0) parent_inner[j] = less(pi);
    const int2 c = children[j], r = range[j];
    children[j] = make_int2(ref(c.x), ref(c.y));
    range[j] = make_int2(less(r.x), less(r.y));
}

// The node of position j among the level's large nodes (sorted by first position), or -1.
__device__ __forceinline__ int task_of_pos(const sah_task *tasks, int cnt, int j) {
    int lo = 0, hi = cnt - 1, k = -1;
    while (lo <= hi) {
        const int mid = (lo + hi) >> 1;
        if (tasks[mid].m.y <= j) {
            k = mid;
            lo = mid + 1;
        } else {
            hi = mid - 1;
        }
    }
    if (k >= 0 && j >= tasks[k].m.z) k = -1;
    return k;
}

// Per position: its node, its interval, and the interval's count and box. A block whose
// positions all lie in one node (most blocks of the top levels, where one node holds many
// blocks' worth) accumulates in shared memory and adds each interval it touched to the global
// bins once; other blocks add every position to the global bins. Counts, minima and maxima do
// not depend on the order of the additions, so the bins are the same either way.
__global__ void __launch_bounds__(kT) k_sah_bin(const sah_task *__restrict__ tasks, const int *__restrict__ n_tasks,
                                                const uint32_t *__restrict__ idx, const float4 *__restrict__ plo,
                                                const float4 *__restrict__ phi, int n, int planes, int32_t *task_of,
                                                uint16_t *binpos, sah_bin *bins) {
    __shared__ uint32_t s_cnt[kMaxSahPlanes + 1], s_lo[3][kMaxSahPlanes + 1], s_hi[3][kMaxSahPlanes + 1];
    __shared__ int s_task;
    const int j0 = blockIdx.x * blockDim.x;
    const int j = j0 + threadIdx.x;
    const int cnt = *n_tasks;
    if (threadIdx.x == 0) {
        const int jl = min(j0 + (int)blockDim.x, n) - 1;
        const int k0 = task_of_pos(tasks, cnt, j0), k1 = task_of_pos(tasks, cnt, jl);
        s_task = (k0 >= 0 && k0 == k1) ? k0 : -1;
    }
    for (int b = threadIdx.x; b <= kMaxSahPlanes; b += blockDim.x) {
        s_cnt[b] = 0u;
        s_lo[0][b] = s_lo[1][b] = s_lo[2][b] = kFull;
        s_hi[0][b] = s_hi[1][b] = s_hi[2][b] = 0u;
    }
    __syncthreads();
    const int local = s_task;
    int k = -1;
    if (j < n) {
        k = local >= 0 ? local : task_of_pos(tasks, cnt, j);
        task_of[j] = k;
    }
    if (k >= 0) {
        const sah_task t = tasks[k];
        const float surf = surface_rn(t.lo.x, t.lo.y, t.lo.z, t.hi.x, t.hi.y, t.hi.z);
        if (surf > 0.f) {  // otherwise the node is split at the median, with no bins
            const int m = t.m.z - t.m.y, P = min(planes, m);
            const int ax = major_axis(t.lo.x, t.lo.y, t.lo.z, t.hi.x, t.hi.y, t.hi.z);
            const float blo = comp(t.lo, ax), q = __fdiv_rn(__fsub_rn(comp(t.hi, ax), blo), (float)(P + 1));
            const uint32_t p = idx[j];
            const float4 l = plo[p], h = phi[p];
            const int b = bin_of(centre(comp(l, ax), comp(h, ax)), blo, q, P);
            binpos[j] = (uint16_t)b;
            if (local >= 0) {
                atomicAdd(&s_cnt[b], 1u);
                atomicMin(&s_lo[0][b], ordered(l.x));
                atomicMin(&s_lo[1][b], ordered(l.y));
                atomicMin(&s_lo[2][b], ordered(l.z));
                atomicMax(&s_hi[0][b], ordered(h.x));
                atomicMax(&s_hi[1][b], ordered(h.y));
                atomicMax(&s_hi[2][b], ordered(h.z));
            } else {
                sah_bin *B = bins + (size_t)t.m.y + k + b;
                atomicAdd(&B->cnt, 1u);
                atomicMin(&B->lo[0], ordered(l.x));
                atomicMin(&B->lo[1], ordered(l.y));
                atomicMin(&B->lo[2], ordered(l.z));
                atomicMax(&B->hi[0], ordered(h.x));
                atomicMax(&B->hi[1], ordered(h.y));
                atomicMax(&B->hi[2], ordered(h.z));
            }
        }
    }
    __syncthreads();
    if (local >= 0) {
        const sah_task t = tasks[local];
        const int P = min(planes, t.m.z - t.m.y);
        sah_bin *B = bins + (size_t)t.m.y + local;
        for (int b = threadIdx.x; b <= P; b += blockDim.x) {
            if (s_cnt[b] == 0u) continue;
            atomicAdd(&B[b].cnt, s_cnt[b]);
            atomicMin(&B[b].lo[0], s_lo[0][b]);
            atomicMin(&B[b].lo[1], s_lo[1][b]);
            atomicMin(&B[b].lo[2], s_lo[2][b]);
            atomicMax(&B[b].hi[0], s_hi[0][b]);
            atomicMax(&B[b].hi[1], s_hi[1][b]);
            atomicMax(&B[b].hi[2], s_hi[2][b]);
        }
    }
}

struct box_acc {
    float l[3], h[3];
    uint32_t c;
    __device__ __forceinline__ void clear() {
        l[0] = l[1] = l[2] = __int_as_float(0x7f800000);
        h[0] = h[1] = h[2] = __int_as_float(0xff800000);
        c = 0;
    }
    __device__ __forceinline__ void add(const box_acc &o) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            l[a] = fminf(l[a], o.l[a]);
            h[a] = fmaxf(h[a], o.h[a]);
        }
        c += o.c;
    }
    __device__ __forceinline__ box_acc shfl_up(int d) const {
        box_acc o;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            o.l[a] = __shfl_up_sync(kFull, l[a], d);
            o.h[a] = __shfl_up_sync(kFull, h[a], d);
        }
        o.c = __shfl_up_sync(kFull, c, d);
        return o;
    }
    __device__ __forceinline__ box_acc shfl_down(int d) const {
        box_acc o;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            o.l[a] = __shfl_down_sync(kFull, l[a], d);
            o.h[a] = __shfl_down_sync(kFull, h[a], d);
        }
        o.c = __shfl_down_sync(kFull, c, d);
        return o;
    }
    __device__ __forceinline__ box_acc shfl(int src) const {
        box_acc o;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            o.l[a] = __shfl_sync(kFull, l[a], src);
            o.h[a] = __shfl_sync(kFull, h[a], src);
        }
        o.c = __shfl_sync(kFull, c, src);
        return o;
    }
    __device__ __forceinline__ float surface() const { return surface_rn(l[0], l[1], l[2], h[0], h[1], h[2]); }
};

__device__ __forceinline__ box_acc load_bin(const sah_bin &b) {
    box_acc a;
    a.c = b.cnt;
    if (a.c == 0) {
        a.clear();
        return a;
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        a.l[k] = unordered(b.lo[k]);
        a.h[k] = unordered(b.hi[k]);
    }
    return a;
}

// (A_l / A) n_l + (A_r / A) n_r, rounded as bvh-ctor.h:449-450 rounds it
__device__ __forceinline__ float split_cost(float al, uint32_t nl, float ar, uint32_t nr, float surf) {
    return __fadd_rn(__fmul_rn(__fdiv_rn(al, surf), (float)nl), __fmul_rn(__fdiv_rn(ar, surf), (float)nr));
}

// One warp per large node: the running boxes of its intervals from the right (kept in shared
// memory) and from the left (carried chunk by chunk), the cost of every plane, the least one.
// The intervals are cleared for the next round as they are read.
__global__ void __launch_bounds__(32 * kChooseWarps) k_sah_choose(const sah_task *__restrict__ tasks,
                                                                  const int *__restrict__ n_tasks, int planes,
                                                                  sah_bin *bins, sah_split *splits) {
    __shared__ box_acc s_suf[kChooseWarps][kMaxSahPlanes + 2];
    const int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int k = blockIdx.x * kChooseWarps + wl;
    if (k >= *n_tasks) return;  // uniform per warp
    const sah_task t = tasks[k];
    const int m = t.m.z - t.m.y;
    const float surf = surface_rn(t.lo.x, t.lo.y, t.lo.z, t.hi.x, t.hi.y, t.hi.z);
    sah_split out;
    out.llo = out.rlo = t.lo;
    out.lhi = out.rhi = t.hi;
    out.m = make_int4(1, 0, m / 2, 0);  // the median of the positions: flat boxes, or no plane separates
    if (surf > 0.f) {
        const int P = min(planes, m), nb = P + 1;
        sah_bin *B = bins + (size_t)t.m.y + k;
        box_acc *suf = s_suf[wl];
        // suffix unions: suf[b] = intervals b .. P
        box_acc carry;
        carry.clear();
        for (int c0 = ((nb - 1) / 32) * 32; c0 >= 0; c0 -= 32) {
            const int b = c0 + lane;
            box_acc v;
            if (b < nb)
                v = load_bin(B[b]);
            else
                v.clear();
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const box_acc o = v.shfl_down(d);
                if (lane + d < 32) v.add(o);
            }
            v.add(carry);
            if (b < nb) suf[b] = v;
            carry = v.shfl(0);
        }
        __syncwarp();
        // prefix unions and the cost of plane b (left: intervals 0 .. b, right: b + 1 .. P)
        carry.clear();
        float best = __int_as_float(0x7f800000);
        int best_i = INT_MAX;
        box_acc best_l, best_r;
        best_l.clear();
        best_r.clear();
        for (int c0 = 0; c0 < nb; c0 += 32) {
            const int b = c0 + lane;
            box_acc v;
            if (b < nb) {
                v = load_bin(B[b]);
                B[b] = sah_bin{0u, {kFull, kFull, kFull}, {0u, 0u, 0u}, 0u};
            } else {
                v.clear();
            }
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const box_acc o = v.shfl_up(d);
                if (lane >= d) v.add(o);
            }
            v.add(carry);
            if (b < P) {
                const box_acc &r = suf[b + 1];
                if (v.c > 0 && r.c > 0) {
                    const float cost = split_cost(v.surface(), v.c, r.surface(), r.c, surf);
                    if (cost < best) {  // ascending b per lane: the first of equal costs stays
                        best = cost;
                        best_i = b;
                        best_l = v;
                        best_r = r;
                    }
                }
            }
            carry = v.shfl(31);
        }
        // least cost over the warp, the lower plane on ties
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) {
            const float oc = __shfl_xor_sync(kFull, best, d);
            const int oi = __shfl_xor_sync(kFull, best_i, d);
            if (oc < best || (oc == best && oi < best_i)) {
                best = oc;
                best_i = oi;
            }
        }
        // plane b was evaluated by lane b % 32, which kept the boxes of its own least plane; the
        // warp's least (cost, plane) is that lane's own least, so its boxes are the winner's
        if (best_i != INT_MAX) {
            const int src = best_i & 31;
            const box_acc L = best_l.shfl(src), R = best_r.shfl(src);
            out.llo = make_float4(L.l[0], L.l[1], L.l[2], 0.f);
            out.lhi = make_float4(L.h[0], L.h[1], L.h[2], 0.f);
            out.rlo = make_float4(R.l[0], R.l[1], R.l[2], 0.f);
            out.rhi = make_float4(R.h[0], R.h[1], R.h[2], 0.f);
            out.m = make_int4(0, best_i, (int)L.c, 0);
        }
    }
    if (lane == 0) splits[k] = out;
}

// left flag of every position of a large node
__global__ void __launch_bounds__(kT) k_sah_flags(const sah_task *__restrict__ tasks,
                                                  const sah_split *__restrict__ splits,
                                                  const int32_t *__restrict__ task_of,
                                                  const uint16_t *__restrict__ binpos, int n, int32_t *flag) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const int k = task_of[j];
    int f = 0;
    if (k >= 0) {
        const int4 sm = splits[k].m;
        f = sm.x ? (j - tasks[k].m.y < sm.z) : ((int)binpos[j] <= sm.y);
    }
    flag[j] = f;
}

// stable partition of every large node's positions; other positions are copied
__global__ void __launch_bounds__(kT) k_sah_scatter(const sah_task *__restrict__ tasks,
                                                    const sah_split *__restrict__ splits,
                                                    const int32_t *__restrict__ task_of,
                                                    const int32_t *__restrict__ flag,
                                                    const int32_t *__restrict__ excl,
                                                    const uint32_t *__restrict__ in, int n, uint32_t *out) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const int k = task_of[j];
    const uint32_t v = in[j];
    if (k < 0) {
        out[j] = v;
        return;
    }
    const int s = tasks[k].m.y, nl = splits[k].m.z;
    const int before = excl[j] - excl[s];
    out[flag[j] ? s + before : s + nl + (j - s - before)] = v;
}

// Writes one split into the tree arrays; returns the two children as tasks.
__device__ __forceinline__ void emit_node(int id, int s, int e, int nl, int2 *children, int2 *range,
                                          int32_t *parent_inner, int32_t *parent_leaf) {
    const int nr = e - s - nl, lid = id + 1, rid = id + nl;
    children[id] = make_int2(nl == 1 ? ~s : lid, nr == 1 ? ~(s + nl) : rid);
    range[id] = make_int2(s, e - 1);
    if (nl == 1)
        parent_leaf[s] = id;
    else
        parent_inner[lid] = id;
    if (nr == 1)
        parent_leaf[s + nl] = id;
    else
        parent_inner[rid] = id;
}

// One thread per large node (and per capacity slot, so that every staging flag is written): the
// node into the tree arrays, its large children staged in position order, its small children
// listed for the warp phase.
__global__ void __launch_bounds__(kT) k_sah_children(const sah_task *__restrict__ tasks,
                                                     const int *__restrict__ n_tasks,
                                                     const sah_split *__restrict__ splits, int cap,
                                                     int2 *children, int2 *range, int32_t *parent_inner,
                                                     int32_t *parent_leaf, sah_task *stage, int32_t *sflag,
                                                     sah_task *small, int *n_small) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= cap) return;
    if (k >= *n_tasks) {
        sflag[2 * k] = sflag[2 * k + 1] = 0;
        return;
    }
    const sah_task t = tasks[k];
    const sah_split sp = splits[k];
    const int id = t.m.x, s = t.m.y, e = t.m.z, nl = sp.m.z, nr = e - s - nl;
    emit_node(id, s, e, nl, children, range, parent_inner, parent_leaf);
    sah_task c[2];
    c[0].lo = sp.llo;
    c[0].hi = sp.lhi;
    c[0].m = make_int4(id + 1, s, s + nl, 0);
    c[1].lo = sp.rlo;
    c[1].hi = sp.rhi;
    c[1].m = make_int4(id + nl, s + nl, e, 0);
    const int sz[2] = {nl, nr};
#pragma unroll
    for (int side = 0; side < 2; ++side) {
        stage[2 * k + side] = c[side];
        sflag[2 * k + side] = sz[side] > kSmall ? 1 : 0;
        if (sz[side] >= 2 && sz[side] <= kSmall) small[atomicAdd(n_small, 1)] = c[side];
    }
}

// the staged large children, in order, as the next round's list
__global__ void __launch_bounds__(kT) k_sah_compact(const sah_task *__restrict__ stage,
                                                    const int32_t *__restrict__ sflag,
                                                    const int32_t *__restrict__ sexcl, int slots, sah_task *next,
                                                    int *n_next) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= slots) return;
    if (sflag[i]) next[sexcl[i]] = stage[i];
    if (i == slots - 1) *n_next = sexcl[i] + sflag[i];
}

// One warp per small node (2 .. kSmall primitives): the subtree, split after split, with the
// primitives in shared memory (slot = position - first) and a stack of ranges still to split.
__global__ void __launch_bounds__(32 * kSmallWarps) k_sah_small(const sah_task *__restrict__ tasks,
                                                                const int *__restrict__ n_tasks, uint32_t *idx,
                                                                const float4 *__restrict__ plo,
                                                                const float4 *__restrict__ phi, int planes,
                                                                int2 *children, int2 *range, int32_t *parent_inner,
                                                                int32_t *parent_leaf, int32_t *info) {
    __shared__ float s_c[kSmallWarps][3][32], s_lo[kSmallWarps][3][32], s_hi[kSmallWarps][3][32];
    __shared__ uint32_t s_idx[kSmallWarps][32];
    __shared__ int3 s_stack[kSmallWarps][32];
    const int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int w = blockIdx.x * kSmallWarps + wl;
    if (w >= *n_tasks) return;  // uniform per warp
    const sah_task t = tasks[w];
    const int s = t.m.y, m = t.m.z - t.m.y;
    if (m < 2 || m > kSmall) {
        if (lane == 0) atomicOr(info + GB_ERR, GB_ERR_TREE);
        return;
    }
    if (lane < m) {
        const uint32_t p = idx[s + lane];
        const float4 l = plo[p], h = phi[p];
        s_idx[wl][lane] = p;
        s_lo[wl][0][lane] = l.x;
        s_lo[wl][1][lane] = l.y;
        s_lo[wl][2][lane] = l.z;
        s_hi[wl][0][lane] = h.x;
        s_hi[wl][1][lane] = h.y;
        s_hi[wl][2][lane] = h.z;
        s_c[wl][0][lane] = centre(l.x, h.x);
        s_c[wl][1][lane] = centre(l.y, h.y);
        s_c[wl][2][lane] = centre(l.z, h.z);
    }
    if (lane == 0) s_stack[wl][0] = make_int3(0, m, t.m.x);
    __syncwarp();
    const float inf = __int_as_float(0x7f800000), ninf = __int_as_float(0xff800000);
    int sp = 1, splits_made = 0;
    while (sp > 0 && splits_made < kSmall) {
        const int3 r = s_stack[wl][--sp];
        __syncwarp();
        const int a = r.x, b = r.y, nid = r.z, mm = b - a;
        const bool in = lane >= a && lane < b;
        float c3[3], l3[3], h3[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            c3[k] = s_c[wl][k][lane];
            l3[k] = s_lo[wl][k][lane];
            h3[k] = s_hi[wl][k][lane];
        }
        const uint32_t my_idx = s_idx[wl][lane];
        // the range's box
        float bl[3], bh[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            bl[k] = in ? l3[k] : inf;
            bh[k] = in ? h3[k] : ninf;
#pragma unroll
            for (int d = 16; d > 0; d >>= 1) {
                bl[k] = fminf(bl[k], __shfl_xor_sync(kFull, bl[k], d));
                bh[k] = fmaxf(bh[k], __shfl_xor_sync(kFull, bh[k], d));
            }
        }
        const int ax = major_axis(bl[0], bl[1], bl[2], bh[0], bh[1], bh[2]);
        const float surf = surface_rn(bl[0], bl[1], bl[2], bh[0], bh[1], bh[2]);
        const float cme = c3[ax];
        // rank of this lane's centre in the range: order-preserving key, then slot (a total
        // order, so that the median split takes exactly mm / 2)
        int rank = 0;
        {
            const uint32_t key = ordered(cme);
            for (int k = a; k < b; ++k) {
                const uint32_t ok = ordered(s_c[wl][ax][k]);
                rank += (ok < key || (ok == key && k < lane)) ? 1 : 0;
            }
        }
        const bool med_left = rank < mm / 2;
        float best = inf;
        int best_i = INT_MAX;  // a plane, or the first degenerate plane for the median
        bool best_med = true;
        float my_plane = 0.f;
        if (surf > 0.f) {
            const int P = min(planes, mm);
            const float blo = bl[ax], q = __fdiv_rn(__fsub_rn(bh[ax], blo), (float)(P + 1));
            my_plane = plane_at(blo, q, lane);
            box_acc L, R;
            L.clear();
            R.clear();
            if (lane < P) {
                for (int k = a; k < b; ++k) {
                    const bool lft = s_c[wl][ax][k] <= my_plane;
#pragma unroll
                    for (int x = 0; x < 3; ++x) {
                        const float lo = s_lo[wl][x][k], hi = s_hi[wl][x][k];
                        L.l[x] = lft ? fminf(L.l[x], lo) : L.l[x];
                        L.h[x] = lft ? fmaxf(L.h[x], hi) : L.h[x];
                        R.l[x] = lft ? R.l[x] : fminf(R.l[x], lo);
                        R.h[x] = lft ? R.h[x] : fmaxf(R.h[x], hi);
                    }
                    L.c += lft ? 1u : 0u;
                    R.c += lft ? 0u : 1u;
                }
            }
            const bool degen = lane < P && (L.c == 0 || R.c == 0);
            float cost = inf;
            int ci = INT_MAX;
            if (lane < P && !degen) {
                const float cc = split_cost(L.surface(), L.c, R.surface(), R.c, surf);
                if (cc < inf) {  // not NaN
                    cost = cc;
                    ci = lane;
                }
            }
#pragma unroll
            for (int d = 16; d > 0; d >>= 1) {
                const float oc = __shfl_xor_sync(kFull, cost, d);
                const int oi = __shfl_xor_sync(kFull, ci, d);
                if (oc < cost || (oc == cost && oi < ci)) {
                    cost = oc;
                    ci = oi;
                }
            }
            best = cost;
            best_i = ci;
            best_med = ci == INT_MAX;
            const unsigned dmask = __ballot_sync(kFull, degen);
            if (dmask) {  // the median split, a candidate in place of the first degenerate plane
                const int at = __ffs(dmask) - 1;
                box_acc ML, MR;
                ML.clear();
                MR.clear();
#pragma unroll
                for (int x = 0; x < 3; ++x) {
                    if (in && med_left) {
                        ML.l[x] = l3[x];
                        ML.h[x] = h3[x];
                    }
                    if (in && !med_left) {
                        MR.l[x] = l3[x];
                        MR.h[x] = h3[x];
                    }
                }
#pragma unroll
                for (int x = 0; x < 3; ++x) {
#pragma unroll
                    for (int d = 16; d > 0; d >>= 1) {
                        ML.l[x] = fminf(ML.l[x], __shfl_xor_sync(kFull, ML.l[x], d));
                        ML.h[x] = fmaxf(ML.h[x], __shfl_xor_sync(kFull, ML.h[x], d));
                        MR.l[x] = fminf(MR.l[x], __shfl_xor_sync(kFull, MR.l[x], d));
                        MR.h[x] = fmaxf(MR.h[x], __shfl_xor_sync(kFull, MR.h[x], d));
                    }
                }
                const int nl = mm / 2;
                const float mc = split_cost(ML.surface(), (uint32_t)nl, MR.surface(), (uint32_t)(mm - nl), surf);
                if (mc < best || (mc == best && at < best_i)) {
                    best = mc;
                    best_i = at;
                    best_med = true;
                }
            }
        }
        const float cut = __shfl_sync(kFull, my_plane, best_med ? 0 : best_i);
        const bool go_left = best_med ? med_left : (cme <= cut);
        const unsigned lm = __ballot_sync(kFull, in && go_left), rm = __ballot_sync(kFull, in && !go_left);
        const int nl = __popc(lm);
        const unsigned below = (1u << lane) - 1u;
        const int slot = go_left ? a + __popc(lm & below) : a + nl + __popc(rm & below);
        __syncwarp();
        if (in) {
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                s_c[wl][k][slot] = c3[k];
                s_lo[wl][k][slot] = l3[k];
                s_hi[wl][k][slot] = h3[k];
            }
            s_idx[wl][slot] = my_idx;
        }
        const int nr = mm - nl;
        if (nl < 1 || nr < 1) {  // cannot happen: every candidate leaves both sides non-empty
            if (lane == 0) atomicOr(info + GB_ERR, GB_ERR_TREE);
            return;
        }
        if (lane == 0) {
            emit_node(nid, s + a, s + b, nl, children, range, parent_inner, parent_leaf);
            int top = sp;
            if (nr >= 2) s_stack[wl][top++] = make_int3(a + nl, b, nid + nl);
            if (nl >= 2) s_stack[wl][top++] = make_int3(a, a + nl, nid + 1);
        }
        sp += (nr >= 2 ? 1 : 0) + (nl >= 2 ? 1 : 0);
        ++splits_made;
        __syncwarp();
    }
    if (sp > 0 && lane == 0) atomicOr(info + GB_ERR, GB_ERR_TREE);
    if (lane < m) idx[s + lane] = s_idx[wl][lane];
}

inline size_t up256(size_t b) { return (b + 255) & ~(size_t)255; }

struct sah_arena {
    uint32_t *idx_a, *idx_b;
    int32_t *task_of, *sflag, *sexcl;
    uint16_t *binpos;
    sah_bin *bins;
    sah_task *tasks_a, *tasks_b, *stage, *small;
    sah_split *splits;
    int *counters;  // large count (two buffers), small count
    int cap;
    size_t nbins, total;
};

sah_arena sah_carve(void *base, uint32_t n) {
    sah_arena A{};
    char *p = (char *)base;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        void *r = p ? p + off : nullptr;
        off += up256(bytes);
        return r;
    };
    const size_t m = n > 0 ? n : 1;
    A.cap = (int)(m / (kSmall + 1) + 1);
    A.nbins = m + (size_t)A.cap + 1;
    A.idx_a = (uint32_t *)take(m * 4);
    A.idx_b = (uint32_t *)take(m * 4);
    A.task_of = (int32_t *)take(m * 4);
    A.binpos = (uint16_t *)take(m * 2);
    A.bins = (sah_bin *)take(A.nbins * sizeof(sah_bin));
    A.tasks_a = (sah_task *)take((size_t)A.cap * sizeof(sah_task));
    A.tasks_b = (sah_task *)take((size_t)A.cap * sizeof(sah_task));
    A.stage = (sah_task *)take(2 * (size_t)A.cap * sizeof(sah_task));
    A.sflag = (int32_t *)take(2 * (size_t)A.cap * 4);
    A.sexcl = (int32_t *)take(2 * (size_t)A.cap * 4);
    A.splits = (sah_split *)take((size_t)A.cap * sizeof(sah_split));
    A.small = (sah_task *)take((m / 2 + 1) * sizeof(sah_task));
    A.counters = (int *)take(4 * sizeof(int));
    A.total = off;
    return A;
}

// The levels of large nodes, from the list the root kernel made, then the warp-per-node phase;
// *order receives the primitive order.
cudaError_t sah_levels(const sah_arena &A, uint32_t n, int planes, const float4 *plo, const float4 *phi,
                       int2 *children, int2 *range, int32_t *parent_inner, int32_t *parent_leaf, int32_t *flag,
                       int32_t *excl, void *cub_tmp, size_t cub_bytes, const uint32_t **order, int32_t *info,
                       cudaStream_t st) {
    const unsigned nb = (n + kT - 1) / kT;
    int *n_large[2] = {A.counters, A.counters + 1}, *n_small = A.counters + 2;
    sah_task *tasks[2] = {A.tasks_a, A.tasks_b};
    uint32_t *idx[2] = {A.idx_a, A.idx_b};
    cudaError_t e = cudaGetLastError();
    int cur = 0;
    // every round takes at least one primitive off each large node, so n rounds always finish
    const int max_rounds = (int)n;
    for (int round = 0; e == cudaSuccess; ++round) {
        if (round % 4 == 3 || round >= max_rounds) {  // stop once no large node is left
            int32_t *left = readback_word();
            e = cudaMemcpyAsync(left, n_large[cur], sizeof(int32_t), cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            if (e != cudaSuccess || *left == 0) break;
            if (round >= max_rounds) return cudaErrorInvalidValue;
        }
        k_sah_bin<<<nb, kT, 0, st>>>(tasks[cur], n_large[cur], idx[cur], plo, phi, (int)n, planes, A.task_of,
                                     A.binpos, A.bins);
        k_sah_choose<<<(A.cap + kChooseWarps - 1) / kChooseWarps, 32 * kChooseWarps, 0, st>>>(
            tasks[cur], n_large[cur], planes, A.bins, A.splits);
        k_sah_flags<<<nb, kT, 0, st>>>(tasks[cur], A.splits, A.task_of, A.binpos, (int)n, flag);
        size_t cb = cub_bytes;
        e = cub::DeviceScan::ExclusiveSum(cub_tmp, cb, flag, excl, (int)n, st);
        if (e != cudaSuccess) break;
        k_sah_scatter<<<nb, kT, 0, st>>>(tasks[cur], A.splits, A.task_of, flag, excl, idx[cur], (int)n,
                                         idx[cur ^ 1]);
        k_sah_children<<<(A.cap + kT - 1) / kT, kT, 0, st>>>(tasks[cur], n_large[cur], A.splits, A.cap, children,
                                                             range, parent_inner, parent_leaf, A.stage, A.sflag,
                                                             A.small, n_small);
        cb = cub_bytes;
        e = cub::DeviceScan::ExclusiveSum(cub_tmp, cb, A.sflag, A.sexcl, 2 * A.cap, st);
        if (e != cudaSuccess) break;
        k_sah_compact<<<(2 * A.cap + kT - 1) / kT, kT, 0, st>>>(A.stage, A.sflag, A.sexcl, 2 * A.cap,
                                                                tasks[cur ^ 1], n_large[cur ^ 1]);
        cur ^= 1;
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) return e;
    k_sah_small<<<(unsigned)((n / 2 + 1 + kSmallWarps - 1) / kSmallWarps), 32 * kSmallWarps, 0, st>>>(
        A.small, n_small, idx[cur], plo, phi, planes, children, range, parent_inner, parent_leaf, info);
    *order = idx[cur];
    return cudaGetLastError();
}

}  // namespace

size_t sah_scratch_bytes(uint32_t n) { return sah_carve(nullptr, n).total; }

cudaError_t sah_tree(void *scratch, uint32_t n, int planes, const float4 *plo, const float4 *phi,
                     const uint32_t *bounds, int2 *children, int2 *range, int32_t *parent_inner,
                     int32_t *parent_leaf, int32_t *flag, int32_t *excl, void *cub_tmp, size_t cub_bytes,
                     const uint32_t **order, int32_t *info, cudaStream_t st) {
    if (n < 2 || planes < 1 || planes > kMaxSahPlanes) return cudaErrorInvalidValue;
    const sah_arena A = sah_carve(scratch, n);
    k_sah_clear<<<(unsigned)((A.nbins + kT - 1) / kT), kT, 0, st>>>(A.bins, A.nbins);
    k_iota<<<(n + kT - 1) / kT, kT, 0, st>>>(A.idx_a, n);
    k_sah_root<<<1, 32, 0, st>>>(bounds, (int)n, A.tasks_a, A.counters, A.small, A.counters + 2);
    return sah_levels(A, n, planes, plo, phi, children, range, parent_inner, parent_leaf, flag, excl, cub_tmp,
                      cub_bytes, order, info, st);
}

cudaError_t sah_tree_set(void *scratch, uint32_t n, const sah_set_scene *scenes, uint32_t count, int planes,
                         const float4 *plo, const float4 *phi, const uint32_t *cbounds, int2 *children,
                         int2 *range, int32_t *parent_inner, int32_t *parent_leaf, int32_t *flag, int32_t *excl,
                         void *cub_tmp, size_t cub_bytes, const uint32_t **order, int32_t *info, cudaStream_t st) {
    if (n < 2 || count == 0 || planes < 1 || planes > kMaxSahPlanes) return cudaErrorInvalidValue;
    const sah_arena A = sah_carve(scratch, n);
    k_sah_clear<<<(unsigned)((A.nbins + kT - 1) / kT), kT, 0, st>>>(A.bins, A.nbins);
    k_iota<<<(n + kT - 1) / kT, kT, 0, st>>>(A.idx_a, n);
    k_sah_roots<<<1, 32, 0, st>>>(scenes, (int)count, cbounds, A.tasks_a, A.counters, A.small, A.counters + 2);
    cudaError_t e = sah_levels(A, n, planes, plo, phi, children, range, parent_inner, parent_leaf, flag, excl,
                               cub_tmp, cub_bytes, order, info, st);
    if (e != cudaSuccess) return e;
    k_sah_localize<<<(n + kT - 1) / kT, kT, 0, st>>>(scenes, (int)count, (int)n, children, range, parent_inner,
                                                     parent_leaf, const_cast<uint32_t *>(*order));
    return cudaGetLastError();
}

}  // namespace grt
