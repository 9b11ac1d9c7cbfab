// Diffuse multi-bounce path tracing and shadow-ray setup on top of the traversal kernels.
//
// The reference wires a diffuse bounce as wavefront steps: find closest hits, then a
// sampling kernel that turns every hit into the next ray (k::sample_cos_dir,
// rt/cuda/bounce.cu:91-142), then find closest hits again. Two forms are implemented:
//   * GRT_PT_WAVEFRONT — that structure, one thread per ray: per bounce a traversal kernel over
//     the queue of live paths and a shade kernel that shades, applies Russian roulette,
//     samples the next direction and appends the survivors to the next queue;
//   * GRT_PT_FUSED — one persistent kernel in which a warp's lanes take paths from a global
//     counter, and each lane traverses, shades and regenerates its path's rays in registers
//     until the path ends, then takes the next path; lanes are refilled whenever too few of
//     a warp's lanes are still busy.
// Both produce the same per-path results: the math is shared (pt_math.cuh) and each path's
// random stream depends only on its index.
#include <algorithm>
#include <mutex>

#include "pathtrace.hpp"
#include "pt_math.cuh"
#include "traverse.cuh"

namespace grt {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kTile = 2048;  // elements per block in the stable compaction

// ---- stable compaction of valid hits (pixel order is kept) ---------------------------------

__device__ __forceinline__ bool hit_valid(const grt_hit *hits, uint32_t i) { return hits[i].t != FLT_MAX; }

__global__ void k_count_valid(const grt_hit *__restrict__ hits, uint32_t n, uint32_t *block_counts) {
    __shared__ uint32_t warp_sums[32];
    const uint32_t base = blockIdx.x * kTile;
    uint32_t c = 0;
    for (uint32_t k = threadIdx.x; k < kTile; k += blockDim.x) {
        const uint32_t i = base + k;
        c += (i < n && hit_valid(hits, i)) ? 1u : 0u;
    }
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(kFull, c, o);
    if ((threadIdx.x & 31) == 0) warp_sums[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t s = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += warp_sums[w];
        block_counts[blockIdx.x] = s;
    }
}

// Exclusive scan of the block counts by one block; writes the total to *total.
__global__ void k_scan_counts(uint32_t *counts, uint32_t nblocks, uint32_t *total) {
    __shared__ uint32_t warp_sums[32];
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (uint32_t base = 0; base < nblocks; base += blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        const uint32_t v = i < nblocks ? counts[i] : 0u;
        uint32_t x = v;  // inclusive warp scan
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(kFull, x, o);
            if ((threadIdx.x & 31) >= (unsigned)o) x += y;
        }
        if ((threadIdx.x & 31) == 31) warp_sums[threadIdx.x >> 5] = x;
        __syncthreads();
        if (threadIdx.x < 32) {
            const uint32_t nw = blockDim.x >> 5;
            uint32_t w = threadIdx.x < nw ? warp_sums[threadIdx.x] : 0u;
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(kFull, w, o);
                if (threadIdx.x >= (unsigned)o) w += y;
            }
            if (threadIdx.x < nw) warp_sums[threadIdx.x] = w;  // inclusive warp prefix
        }
        __syncthreads();
        const uint32_t wid = threadIdx.x >> 5;
        const uint32_t excl = carry + (wid ? warp_sums[wid - 1] : 0u) + x - v;
        if (i < nblocks) counts[i] = excl;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry = excl + v;
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

// Scatter pass: element i with a valid hit goes to out position offset(i). `emit(i, pos)`.
template <typename Emit>
__device__ void scatter_valid(const grt_hit *__restrict__ hits, uint32_t n, const uint32_t *block_offsets, Emit emit) {
    __shared__ uint32_t warp_sums[32];
    __shared__ uint32_t carry;
    const uint32_t base = blockIdx.x * kTile;
    if (threadIdx.x == 0) carry = block_offsets[blockIdx.x];
    __syncthreads();
    const unsigned lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (uint32_t r = 0; r < kTile; r += blockDim.x) {
        const uint32_t i = base + r + threadIdx.x;
        const bool f = i < n && hit_valid(hits, i);
        const unsigned b = __ballot_sync(kFull, f);
        if (lane == 0) warp_sums[wid] = __popc(b);
        __syncthreads();
        uint32_t before = carry;
        for (unsigned w = 0; w < wid; ++w) before += warp_sums[w];
        if (f) emit(i, before + __popc(b & ((1u << lane) - 1u)));
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t s = 0;
            for (unsigned w = 0; w < nw; ++w) s += warp_sums[w];
            carry += s;
        }
        __syncthreads();
    }
}

__global__ void k_scatter_indices(const grt_hit *__restrict__ hits, uint32_t n, const uint32_t *block_offsets,
                                  uint32_t *out) {
    scatter_valid(hits, n, block_offsets, [&](uint32_t i, uint32_t pos) { out[pos] = i; });
}

__device__ __forceinline__ pm::f3 vtx(const float4 *__restrict__ v, uint32_t i) {
    const float4 p = __ldg(v + i);
    return {p.x, p.y, p.z};
}

// Facing geometric normal of triangle `ref` for a ray travelling along d.
__device__ __forceinline__ pm::f3 tri_normal(const pt_scene &ps, uint32_t ref, pm::f3 d, uint32_t &material) {
    const uint4 t = __ldg(ps.tris + ref);
    material = t.w;
    return pm::facing_normal(vtx(ps.vpos, t.x), vtx(ps.vpos, t.y), vtx(ps.vpos, t.z), d);
}

__global__ void k_scatter_shadow(const grt_hit *__restrict__ hits, uint32_t n, const uint32_t *block_offsets,
                                 const float4 *__restrict__ rays, pt_scene ps, float lx, float ly, float lz, float eps,
                                 float4 *out) {
    scatter_valid(hits, n, block_offsets, [&](uint32_t i, uint32_t pos) {
        const float4 a = rays[2 * (size_t)i], b = rays[2 * (size_t)i + 1];
        const pm::f3 o = {a.x, a.y, a.z}, d = {b.x, b.y, b.z};
        uint32_t m;
        const pm::f3 nrm = tri_normal(ps, hits[i].ref, d, m);
        const pm::f3 p = pm::offset_hit_point(o, d, hits[i].t, nrm, eps);
        const pm::f3 to = pm::sub3({lx, ly, lz}, p);
        const float dist = pm::sqrt_rn(pm::dot3(to, to));
        const pm::f3 dir = {pm::div(to.x, dist), pm::div(to.y, dist), pm::div(to.z, dist)};
        out[2 * (size_t)pos] = make_float4(p.x, p.y, p.z, eps);
        out[2 * (size_t)pos + 1] = make_float4(dir.x, dir.y, dir.z, pm::sub(dist, eps));
    });
}

// ---- path state and the per-bounce logic shared by both forms -------------------------------

struct path_t {
    pm::pcg32 rng;
    float thr;        // throughput
    uint32_t digest;  // running digest of the path's hits
    uint32_t bounce;  // index of the bounce ray currently traced (1-based)
    uint32_t last_ref;
};

// Path state of the fused kernel, kept in shared memory next to the traversal stacks (one
// structure-of-arrays slot per thread) because only the shade phase touches it; the PCG32
// increment is recomputed from the path index.
struct path_slots {
    uint64_t *rng;
    float *thr;
    uint32_t *digest, *bounce, *last_ref, *path;
};

__device__ __forceinline__ path_slots path_slots_at(int *smem_base, int stack_entries) {
    const int bt = blockDim.x;
    char *base = reinterpret_cast<char *>(smem_base + (size_t)stack_entries * bt);
    path_slots ps;
    ps.rng = reinterpret_cast<uint64_t *>(base);
    ps.thr = reinterpret_cast<float *>(base + 8 * bt);
    ps.digest = reinterpret_cast<uint32_t *>(base + 12 * bt);
    ps.bounce = reinterpret_cast<uint32_t *>(base + 16 * bt);
    ps.last_ref = reinterpret_cast<uint32_t *>(base + 20 * bt);
    ps.path = reinterpret_cast<uint32_t *>(base + 24 * bt);
    return ps;
}
constexpr int kPathSlotBytes = 28;

__device__ __forceinline__ void path_save(const path_slots &sl, int t, uint32_t p, const path_t &st) {
    sl.rng[t] = st.rng.state;
    sl.thr[t] = st.thr;
    sl.digest[t] = st.digest;
    sl.bounce[t] = st.bounce;
    sl.last_ref[t] = st.last_ref;
    sl.path[t] = p;
}

__device__ __forceinline__ uint32_t path_load(const path_slots &sl, int t, uint64_t seed, path_t &st) {
    const uint32_t p = sl.path[t];
    st.rng.state = sl.rng[t];
    st.rng.inc = ((seed + p) << 1u) | 1u;
    st.thr = sl.thr[t];
    st.digest = sl.digest[t];
    st.bounce = sl.bounce[t];
    st.last_ref = sl.last_ref[t];
    return p;
}

__device__ __forceinline__ float albedo_of(const pt_scene &ps, uint32_t material) {
    return material < ps.n_albedo ? __ldg(ps.albedo + material) : 0.8f;
}

// First bounce ray of path p: from primary hit H[p mod |H|].
__device__ __forceinline__ void path_start(const pt_scene &ps, const pt_params_dev &pp, uint32_t p,
                                           const float4 *__restrict__ prim_rays, const grt_hit *__restrict__ prim_hits,
                                           const uint32_t *__restrict__ hit_list, uint32_t n_list, path_t &st,
                                           float4 &ro, float4 &rd) {
    const uint32_t i = __ldg(hit_list + (p % n_list));
    const float4 a = __ldg(prim_rays + 2 * (size_t)i), b = __ldg(prim_rays + 2 * (size_t)i + 1);
    const float4 h = __ldg(reinterpret_cast<const float4 *>(prim_hits) + i);
    const pm::f3 o = {a.x, a.y, a.z}, d = {b.x, b.y, b.z};
    st.rng.set_sequence((uint64_t)pp.seed + p);
    st.thr = 1.0f;
    st.digest = pm::kDigestSeed;
    st.bounce = 1;
    st.last_ref = pm::kMissWord;
    uint32_t m;
    const pm::f3 n = tri_normal(ps, __float_as_uint(h.w), d, m);
    const pm::f3 org = pm::offset_hit_point(o, d, h.x, n, pp.eps);
    const float u0 = st.rng.uniform(), u1 = st.rng.uniform();
    const pm::f3 dir = pm::align(pm::cosine_sample_hemisphere(u0, u1), n);
    ro = make_float4(org.x, org.y, org.z, pp.eps);
    rd = make_float4(dir.x, dir.y, dir.z, FLT_MAX);
}

// Facing normal and material of a hit from its triangle record (v0, v0 - v1 with the material
// id in w, v0 - v2): cross(v0 - v1, v0 - v2) equals cross(v1 - v0, v2 - v0) bit for bit, because
// a rounded difference negates exactly, so this is the same normal tri_normal computes.
__device__ __forceinline__ pm::f3 record_normal(const float4 *__restrict__ records, uint32_t rec, pm::f3 d,
                                                uint32_t &material) {
    const float4 p1 = __ldg(records + 3 * (size_t)rec + 1), p2 = __ldg(records + 3 * (size_t)rec + 2);
    material = __float_as_uint(p1.w);
    pm::f3 n = pm::normalize3(pm::cross3({p1.x, p1.y, p1.z}, {p2.x, p2.y, p2.z}));
    if (pm::dot3(d, n) > 0.f) n = {-n.x, -n.y, -n.z};
    return n;
}

// Consumes the closest hit of the current bounce ray (o, d). Returns true if the path goes on,
// with (o, d) replaced by the next ray's origin and direction; otherwise fills `res`.
// FROM_RECORD: take normal and material from the hit's triangle record instead of the
// triangle and vertex arrays.
template <bool FROM_RECORD>
__device__ __forceinline__ bool path_bounce(const pt_scene &ps, const float4 *records, const pt_params_dev &pp,
                                            path_t &st, const hit_t &h, pm::f3 &o, pm::f3 &d, grt_path_result &res) {
    if (h.t == FLT_MAX) {  // escaped: collects the sky
        st.digest = pm::digest_word(st.digest, pm::kMissWord);
        res = {pm::mul(st.thr, pm::sky(d)), st.bounce, st.last_ref, st.digest};
        return false;
    }
    st.digest = pm::digest_word(pm::digest_word(st.digest, h.ref), __float_as_uint(h.t));
    st.last_ref = h.ref;
    uint32_t m;
    const pm::f3 n = FROM_RECORD ? record_normal(records, h.rec, d, m) : tri_normal(ps, h.ref, d, m);
    st.thr = pm::mul(st.thr, albedo_of(ps, m));
    if (st.bounce >= pp.max_bounces) {
        res = {0.f, st.bounce, st.last_ref, st.digest};
        return false;
    }
    if (st.bounce + 1 >= pp.rr_start) {  // Russian roulette before the next bounce
        if (!(st.rng.uniform() < pp.rr_continue)) {
            res = {0.f, st.bounce, st.last_ref, st.digest};
            return false;
        }
        st.thr = pm::div(st.thr, pp.rr_continue);
    }
    o = pm::offset_hit_point(o, d, h.t, n, pp.eps);
    const float u0 = st.rng.uniform(), u1 = st.rng.uniform();
    d = pm::align(pm::cosine_sample_hemisphere(u0, u1), n);
    ++st.bounce;
    return true;
}

__device__ __forceinline__ void record_bounce(grt_hit *bounce_hits, const pt_params_dev &pp, uint32_t p,
                                              uint32_t bounce, const hit_t &h) {
    if (bounce_hits)
        reinterpret_cast<float4 *>(bounce_hits)[(size_t)p * pp.max_bounces + (bounce - 1)] =
            make_float4(h.t, h.b, h.g, __uint_as_float(h.ref));
}

__device__ __forceinline__ void clear_unused(grt_hit *bounce_hits, const pt_params_dev &pp, uint32_t p,
                                             uint32_t traced) {
    if (bounce_hits)
        for (uint32_t k = traced; k < pp.max_bounces; ++k)
            reinterpret_cast<float4 *>(bounce_hits)[(size_t)p * pp.max_bounces + k] = make_float4(0.f, 0.f, 0.f, 0.f);
}

__device__ __forceinline__ ray_t make_ray(pm::f3 o, pm::f3 d, float tmin, float tmax) {
    return grt::make_ray(o.x, o.y, o.z, d.x, d.y, d.z, tmin, tmax);
}

// ---- wavefront form -----------------------------------------------------------------------

struct wf_state {
    uint64_t rng_state, rng_inc;
    float thr;
    uint32_t digest, bounce, last_ref;
};

__global__ void k_wf_init(pt_scene ps, pt_params_dev pp, const float4 *__restrict__ prim_rays,
                          const grt_hit *__restrict__ prim_hits, const uint32_t *__restrict__ hit_list,
                          const uint32_t *__restrict__ n_list, uint32_t n_paths, wf_state *states, uint32_t *queue,
                          float4 *rays, grt_path_result *results, uint32_t *n_queue) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p == 0) *n_queue = n_paths;
    if (p >= n_paths) return;
    path_t st;
    float4 ro, rd;
    const uint32_t nl = *n_list;
    if (nl == 0) {  // no primary hit at all: every path is empty
        results[p] = {0.f, 0u, pm::kMissWord, pm::kDigestSeed};
        queue[p] = 0xFFFFFFFFu;
        rays[2 * (size_t)p] = make_float4(0.f, 0.f, 0.f, 1.f);
        rays[2 * (size_t)p + 1] = make_float4(0.f, 0.f, 1.f, -1.f);  // empty interval: misses
        return;
    }
    path_start(ps, pp, p, prim_rays, prim_hits, hit_list, nl, st, ro, rd);
    states[p] = {st.rng.state, st.rng.inc, st.thr, st.digest, st.bounce, st.last_ref};
    queue[p] = p;
    rays[2 * (size_t)p] = ro;
    rays[2 * (size_t)p + 1] = rd;
}

__global__ void k_wf_shade(pt_scene ps, pt_params_dev pp, const uint32_t *__restrict__ n_in,
                           const uint32_t *__restrict__ queue_in, const float4 *__restrict__ rays_in,
                           const grt_hit *__restrict__ hits, wf_state *states, uint32_t *n_out, uint32_t *queue_out,
                           float4 *rays_out, grt_path_result *results, grt_hit *bounce_hits) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = *n_in;
    bool go_on = false;
    uint32_t p = 0;
    float4 ro, rd;
    if (k < n) {
        p = queue_in[k];
        if (p != 0xFFFFFFFFu) {
            wf_state w = states[p];
            path_t st;
            st.rng.state = w.rng_state;
            st.rng.inc = w.rng_inc;
            st.thr = w.thr;
            st.digest = w.digest;
            st.bounce = w.bounce;
            st.last_ref = w.last_ref;
            ro = rays_in[2 * (size_t)k];
            rd = rays_in[2 * (size_t)k + 1];
            const float4 hv = reinterpret_cast<const float4 *>(hits)[k];
            hit_t h = {hv.x, hv.y, hv.z, __float_as_uint(hv.w), 0u};
            record_bounce(bounce_hits, pp, p, st.bounce, h);
            grt_path_result res;
            pm::f3 o = {ro.x, ro.y, ro.z}, d = {rd.x, rd.y, rd.z};
            go_on = path_bounce<false>(ps, nullptr, pp, st, h, o, d, res);
            ro = make_float4(o.x, o.y, o.z, pp.eps);
            rd = make_float4(d.x, d.y, d.z, FLT_MAX);
            if (go_on) {
                states[p] = {st.rng.state, st.rng.inc, st.thr, st.digest, st.bounce, st.last_ref};
            } else {
                results[p] = res;
                clear_unused(bounce_hits, pp, p, st.bounce);
            }
        }
    }
    // warp-aggregated append to the next queue
    const unsigned m = __ballot_sync(kFull, go_on);
    if (m == 0) return;
    const unsigned lane = threadIdx.x & 31;
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(n_out, __popc(m));
    base = __shfl_sync(kFull, base, 0);
    if (go_on) {
        const uint32_t slot = base + __popc(m & ((1u << lane) - 1u));
        queue_out[slot] = p;
        rays_out[2 * (size_t)slot] = ro;
        rays_out[2 * (size_t)slot + 1] = rd;
    }
}

// ---- fused persistent form ----------------------------------------------------------------

// First bounce ray and generator state of every path, launched just before the fused kernel: a
// lane that takes a path then reads 32 coalesced bytes instead of following four dependent
// loads (hit list -> primary ray and hit -> triangle -> vertices) while its warp waits (on
// GB300 this took 2.3 % off the fused launch, the extra kernel included). The paths of one
// primary hit (p = i + |H| m) share its origin and normal, so a thread takes hit-list entry i and
// up to kStartsPerThread of its paths: one chain of dependent loads for all of them.
// starts[2p] = (origin, low word of the PCG32 state after the two direction draws),
// starts[2p + 1] = (direction, high word); t_min = eps, t_max = FLT_MAX for every first ray.
constexpr uint32_t kStartsPerThread = 4;

__global__ void k_pt_starts(pt_scene ps, pt_params_dev pp, const float4 *__restrict__ prim_rays,
                            const grt_hit *__restrict__ prim_hits, const uint32_t *__restrict__ hit_list,
                            const uint32_t *__restrict__ n_list, uint32_t n_paths, float4 *starts) {
    const uint32_t nl = *n_list;
    if (nl == 0) return;
    // thread t: entry li = t mod |H| and its paths li + |H| (kStartsPerThread g + k), g = t / |H|
    const uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    const uint64_t g = t / nl;
    const uint32_t li = (uint32_t)(t - g * nl);
    const uint64_t p0 = li + (uint64_t)nl * g * kStartsPerThread;
    if (p0 >= n_paths) return;
    const uint32_t i = __ldg(hit_list + li);
    const float4 a = __ldg(prim_rays + 2 * (size_t)i), b = __ldg(prim_rays + 2 * (size_t)i + 1);
    const float4 h = __ldg(reinterpret_cast<const float4 *>(prim_hits) + i);
    const pm::f3 o = {a.x, a.y, a.z}, d = {b.x, b.y, b.z};
    uint32_t m;
    const pm::f3 n = tri_normal(ps, __float_as_uint(h.w), d, m);
    const pm::f3 org = pm::offset_hit_point(o, d, h.x, n, pp.eps);
    for (uint32_t k = 0; k < kStartsPerThread; ++k) {
        const uint64_t p = p0 + (uint64_t)nl * k;
        if (p >= n_paths) break;
        pm::pcg32 rng;
        rng.set_sequence((uint64_t)pp.seed + p);  // as path_start
        const float u0 = rng.uniform(), u1 = rng.uniform();
        const pm::f3 dir = pm::align(pm::cosine_sample_hemisphere(u0, u1), n);
        starts[2 * p] = make_float4(org.x, org.y, org.z, __uint_as_float((uint32_t)rng.state));
        starts[2 * p + 1] = make_float4(dir.x, dir.y, dir.z, __uint_as_float((uint32_t)(rng.state >> 32)));
    }
}

// Threads k_pt_starts needs at most for n_paths paths over |H| <= min(n_primary, n_paths) used
// entries: |H| ceil(ceil(n_paths / |H|) / K) <= n_paths / K + 2 |H|.
inline uint64_t starts_threads(uint32_t n_paths, uint32_t n_primary) {
    return (uint64_t)n_paths / kStartsPerThread + 2 * (uint64_t)std::min(n_primary, n_paths) + 1;
}

// Each warp alternates between two phases (a lane takes a new path's first ray from `starts`).
// In the traversal phase the lanes that hold a ray
// run trav_iter; a lane whose ray ends keeps its closest hit and waits. When fewer than
// `refill_threshold` lanes are still traversing, the warp enters the shade phase: all waiting
// lanes shade their hit together (Russian roulette, next bounce direction) and go back to
// traversal, or finish their path and take a new one from the global path counter. Shading and
// path set-up therefore run warp-coherently instead of one lane at a time.
template <int ORDER, bool ALPHA, int FP = 0>
__global__ void __launch_bounds__(256) k_pt_fused(dev_scene sc, pt_scene ps, pt_params_dev pp,
                                                  const float4 *__restrict__ prim_rays,
                                                  const grt_hit *__restrict__ prim_hits,
                                                  const uint32_t *__restrict__ hit_list,
                                                  const uint32_t *__restrict__ n_list, uint32_t n_paths,
                                                  grt_path_result *results, grt_hit *bounce_hits, unsigned *err,
                                                  unsigned *counter, int refill_threshold, int refill_period, int cap,
                                                  spec_cfg spec, const float4 *__restrict__ starts) {
    extern __shared__ int s_stack[];
    if (stop_requested_at_entry(err)) return;  // the host asked the context to stop
    const unsigned lane = threadIdx.x & 31u;
    const unsigned lanes_below = (1u << lane) - 1u;
    int *stk = s_stack + threadIdx.x;
    const int stride = blockDim.x;
    const path_slots slots = path_slots_at(s_stack, cap);
    constexpr bool SPEC = ORDER == SPECULATIVE || ORDER == WIDE_SPECULATIVE;
    constexpr bool WIDE = ORDER == WIDE_SPECULATIVE;
    const int me = threadIdx.x;
    const uint32_t nl = *n_list;
    trav_t s;
    ray_t r;
    bool tracing = false;   // the lane's ray is being traversed
    bool waiting = false;   // the lane's ray has ended and its hit waits to be shaded
    bool plain = false, exhausted = false;
    for (;;) {
        // shade phase: waiting lanes consume their hit
        if (waiting) {
            waiting = false;
            path_t st;
            const uint32_t p = path_load(slots, me, pp.seed, st);
            record_bounce(bounce_hits, pp, p, st.bounce, s.hit);
            pm::f3 o = {r.ox(), r.oy(), r.oz()}, d = {r.dx, r.dy, r.dz};
            grt_path_result res;
            if (path_bounce<true>(ps, sc.records, pp, st, s.hit, o, d, res)) {
                path_save(slots, me, p, st);
                r = make_ray(o, d, pp.eps, FLT_MAX);
                trav_init(s, sc, r, WIDE);
                plain = sc.finite && ray_is_plain(r);
                tracing = true;
            } else {
                results[p] = res;
                clear_unused(bounce_hits, pp, p, st.bounce);
            }
        }
        // refill phase: lanes without a path take the next ones
        if (!exhausted) {
            const unsigned need = __ballot_sync(kFull, !tracing);
            if (need) {
                const unsigned cnt = __popc(need);
                unsigned base = 0;
                if (lane == 0) base = atomicAdd(counter, cnt);
                base = __shfl_sync(kFull, base, 0);
                if (base + cnt >= n_paths) exhausted = true;
                if (!tracing) {
                    const uint32_t my = base + __popc(need & lanes_below);
                    if (my < n_paths) {
                        if (nl == 0) {
                            results[my] = {0.f, 0u, pm::kMissWord, pm::kDigestSeed};
                            clear_unused(bounce_hits, pp, my, 0);
                        } else {
                            const float4 a = __ldg(starts + 2 * (size_t)my), b = __ldg(starts + 2 * (size_t)my + 1);
                            path_t st;
                            st.rng.state = ((uint64_t)__float_as_uint(b.w) << 32) | __float_as_uint(a.w);
                            st.rng.inc = ((pp.seed + my) << 1u) | 1u;
                            st.thr = 1.0f;
                            st.digest = pm::kDigestSeed;
                            st.bounce = 1;
                            st.last_ref = pm::kMissWord;
                            path_save(slots, me, my, st);
                            r = make_ray({a.x, a.y, a.z}, {b.x, b.y, b.z}, pp.eps, FLT_MAX);
                            trav_init(s, sc, r, WIDE);
                            plain = sc.finite && ray_is_plain(r);
                            tracing = true;
                        }
                    }
                }
            }
        }
        if (__ballot_sync(kFull, tracing) == 0) {
            if (exhausted) break;
            continue;
        }
        // traversal phase
        for (int it = 1;; ++it) {
            if (SPEC && __all_sync(kFull, !tracing || plain))  // every ray of the warp plain (nearly always)
                trav_spec_iter<false, false, WIDE, ALPHA, kFastVisits[FP], kFastPend[FP], true>(s, tracing, plain, sc, r,
                                                                                                stk, stride, cap, spec,
                                                                                                err);
            else if (SPEC)
                trav_spec_iter<false, false, WIDE, ALPHA, kFastVisits[FP], kFastPend[FP]>(s, tracing, plain, sc, r, stk,
                                                                                          stride, cap, spec, err);
            else if (tracing && plain)
                trav_advance<ORDER, false, false, true, ALPHA>(s, sc, r, stk, stride, cap, err);
            else if (tracing)
                trav_advance<ORDER, false, false, false, ALPHA>(s, sc, r, stk, stride, cap, err);
            if (tracing && s.done) {
                tracing = false;
                waiting = true;
            }
            if (it % refill_period == 0) {
                const int busy = __popc(__ballot_sync(kFull, tracing));
                if (busy < refill_threshold) break;
            }
        }
    }
}

using fused_fn_t = void (*)(dev_scene, pt_scene, pt_params_dev, const float4 *, const grt_hit *, const uint32_t *,
                           const uint32_t *, uint32_t, grt_path_result *, grt_hit *, unsigned *, unsigned *, int, int,
                           int, spec_cfg, const float4 *);

// The fused kernel instance for the loop order, alpha-aware tracing and fast-path instance `fp`
// (the speculative order without alpha has the instances of kFastVisits / kFastPend).
template <int ORDER> fused_fn_t fused_kernel_of(bool alpha, int fp) {
    if (alpha) return k_pt_fused<ORDER, true>;
    if (ORDER == SPECULATIVE) {
        switch (fp) {
            case 1: return k_pt_fused<ORDER, false, ORDER == SPECULATIVE ? 1 : 0>;
            case 2: return k_pt_fused<ORDER, false, ORDER == SPECULATIVE ? 2 : 0>;
            case 3: return k_pt_fused<ORDER, false, ORDER == SPECULATIVE ? 3 : 0>;
            case 4: return k_pt_fused<ORDER, false, ORDER == SPECULATIVE ? 4 : 0>;
            default: break;
        }
    }
    return k_pt_fused<ORDER, false>;
}

fused_fn_t fused_kernel(int order, bool alpha, int fp) {
    return order == WHILE_WHILE        ? fused_kernel_of<WHILE_WHILE>(alpha, fp)
           : order == SPECULATIVE      ? fused_kernel_of<SPECULATIVE>(alpha, fp)
           : order == WIDE_SPECULATIVE ? fused_kernel_of<WIDE_SPECULATIVE>(alpha, fp)
                                       : fused_kernel_of<IF_IF>(alpha, fp);
}

template <int ORDER>
cudaError_t fused_launch(const dev_scene &sc, const pt_scene &ps, const pt_params_dev &pp, const float4 *prim_rays,
                         const grt_hit *prim_hits, uint32_t n_primary, const uint32_t *hit_list,
                         const uint32_t *n_list, uint32_t n_paths,
                         grt_path_result *results, grt_hit *bounce_hits, const launch_params &lp, unsigned *err,
                         unsigned *counter, float4 *starts, cudaStream_t st) {
    const size_t smem = (size_t)(lp.stack_entries * sizeof(int) + kPathSlotBytes) * lp.block_threads;
    const fused_fn_t kern = fused_kernel_of<ORDER>(sc.alpha != nullptr, fast_path_of(lp.spec));
    cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(unsigned), st);
    if (e != cudaSuccess) return e;
    k_pt_starts<<<(unsigned)((starts_threads(n_paths, n_primary) + 255) / 256), 256, 0, st>>>(
        ps, pp, prim_rays, prim_hits, hit_list, n_list, n_paths, starts);
    kern<<<lp.grid_blocks, lp.block_threads, smem, st>>>(sc, ps, pp, prim_rays, prim_hits, hit_list, n_list, n_paths,
                                                         results, bounce_hits, err, counter, lp.refill_threshold,
                                                         lp.refill_period, lp.stack_entries, lp.spec, starts);
    return cudaGetLastError();
}

}  // namespace

size_t compact_scratch_bytes(uint32_t n) { return (size_t)((n + kTile - 1) / kTile + 1) * sizeof(uint32_t); }

cudaError_t launch_compact_hits(const grt_hit *hits, uint32_t n, uint32_t *out_indices, uint32_t *count,
                                uint32_t *scratch, cudaStream_t st) {
    const uint32_t nb = (n + kTile - 1) / kTile;
    if (nb == 0) return cudaMemsetAsync(count, 0, sizeof(uint32_t), st);
    k_count_valid<<<nb, 256, 0, st>>>(hits, n, scratch);
    k_scan_counts<<<1, 1024, 0, st>>>(scratch, nb, count);
    k_scatter_indices<<<nb, 256, 0, st>>>(hits, n, scratch, out_indices);
    return cudaGetLastError();
}

cudaError_t launch_shadow_rays(const pt_scene &ps, const float4 *rays, const grt_hit *hits, uint32_t n,
                               const float light[3], float eps, float4 *out_rays, uint32_t *count, uint32_t *scratch,
                               cudaStream_t st) {
    const uint32_t nb = (n + kTile - 1) / kTile;
    if (nb == 0) return cudaMemsetAsync(count, 0, sizeof(uint32_t), st);
    k_count_valid<<<nb, 256, 0, st>>>(hits, n, scratch);
    k_scan_counts<<<1, 1024, 0, st>>>(scratch, nb, count);
    k_scatter_shadow<<<nb, 256, 0, st>>>(hits, n, scratch, rays, ps, light[0], light[1], light[2], eps, out_rays);
    return cudaGetLastError();
}

cudaError_t launch_wavefront_init(const pt_scene &ps, const pt_params_dev &pp, const float4 *prim_rays,
                                  const grt_hit *prim_hits, const uint32_t *hit_list, const uint32_t *n_list,
                                  uint32_t n_paths, void *states, uint32_t *queue, float4 *rays,
                                  grt_path_result *results, uint32_t *n_queue, cudaStream_t st) {
    const uint32_t nb = (n_paths + 255) / 256;
    k_wf_init<<<nb, 256, 0, st>>>(ps, pp, prim_rays, prim_hits, hit_list, n_list, n_paths, (wf_state *)states, queue,
                                  rays, results, n_queue);
    return cudaGetLastError();
}

cudaError_t launch_wavefront_shade(const pt_scene &ps, const pt_params_dev &pp, uint32_t max_n, const uint32_t *n_in,
                                   const uint32_t *queue_in, const float4 *rays_in, const grt_hit *hits, void *states,
                                   uint32_t *n_out, uint32_t *queue_out, float4 *rays_out, grt_path_result *results,
                                   grt_hit *bounce_hits, cudaStream_t st) {
    const uint32_t nb = (max_n + 255) / 256;
    k_wf_shade<<<nb, 256, 0, st>>>(ps, pp, n_in, queue_in, rays_in, hits, (wf_state *)states, n_out, queue_out,
                                   rays_out, results, bounce_hits);
    return cudaGetLastError();
}

size_t wavefront_state_bytes() { return sizeof(wf_state); }

cudaError_t launch_fused(const dev_scene &sc, const pt_scene &ps, const pt_params_dev &pp, const float4 *prim_rays,
                         const grt_hit *prim_hits, uint32_t n_primary, const uint32_t *hit_list,
                         const uint32_t *n_list, uint32_t n_paths,
                         grt_path_result *results, grt_hit *bounce_hits, const launch_params &lp, unsigned *err,
                         unsigned *counter, float4 *starts, cudaStream_t st) {
    if (n_paths == 0) return cudaSuccess;
    if (!spec_ok(lp.spec)) return cudaErrorInvalidValue;
    auto f = lp.order == WHILE_WHILE        ? fused_launch<WHILE_WHILE>
             : lp.order == SPECULATIVE      ? fused_launch<SPECULATIVE>
             : lp.order == WIDE_SPECULATIVE ? fused_launch<WIDE_SPECULATIVE>
                                            : fused_launch<IF_IF>;
    return f(sc, ps, pp, prim_rays, prim_hits, n_primary, hit_list, n_list, n_paths, results, bounce_hits, lp, err,
             counter, starts, st);
}

cudaError_t prepare_pt_kernels() {
    const int bytes = (kStackLarge * (int)sizeof(int) + kPathSlotBytes) * 256;
    for (int order : {(int)IF_IF, (int)WHILE_WHILE, (int)SPECULATIVE, (int)WIDE_SPECULATIVE})
        for (int fp = 0; fp <= kFastPaths; ++fp) {  // fp == kFastPaths: the alpha-aware instance
            const void *f = (const void *)fused_kernel(order, fp == kFastPaths, fp == kFastPaths ? 0 : fp);
            cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
            if (e != cudaSuccess) return e;
        }
    return cudaSuccess;
}

int fused_blocks_per_sm(int block_threads, int stack_entries, int order, bool alpha, const spec_cfg &spec) {
    int blocks = 0;
    const size_t smem = (size_t)(stack_entries * sizeof(int) + kPathSlotBytes) * block_threads;
    const void *fn = (const void *)fused_kernel(order, alpha, alpha ? 0 : fast_path_of(spec));
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, fn, block_threads, smem) != cudaSuccess) return 1;
    return blocks > 0 ? blocks : 1;
}

}  // namespace grt

// ---- allocation-free compaction ------------------------------------------------------------
//
// grt_compact_hits_static is grt_compact_hits for callers that must not allocate device
// memory: a renderer that reserves its whole device-memory budget up front and hands out
// memory only from its own pool, or a frame loop that cannot afford cudaMalloc's implicit
// device synchronisation in the middle of a frame. Its only temporary storage, one count per
// 2048-hit tile, lives in the fixed array below, which every GPU that loads this library holds
// until the process exits. The array's device address is looked up once per device and kept
// for the life of the process, so a process that resets a device (cudaDeviceReset) must not
// call this entry point on that device afterwards.

namespace grt {
namespace {

constexpr uint32_t kStaticTiles = 16384;  // 64 KiB of tile counts: up to 16384 * 2048 hits
static_assert((uint64_t)kStaticTiles * kTile == GRT_COMPACT_STATIC_MAX_HITS, "capacity mismatch");

static __device__ __align__(256) uint32_t g_compact_tiles[kStaticTiles];

constexpr int kMaxDevices = 64;
std::mutex g_tiles_mutex;
uint32_t *g_tiles_addr[kMaxDevices] = {};

// Device address of g_compact_tiles on the current device, looked up once per device. In host
// code the symbol itself is only a host-side stand-in, never a device address.
cudaError_t static_tiles(uint32_t **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_tiles_mutex);
    if (!g_tiles_addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_compact_tiles);
        if (e != cudaSuccess) return e;
        g_tiles_addr[dev] = (uint32_t *)p;
    }
    *out = g_tiles_addr[dev];
    return cudaSuccess;
}

}  // namespace
}  // namespace grt

extern "C" grt_status grt_compact_hits_static(const grt_hit *hits_dev, uint32_t n, uint32_t *indices_dev,
                                              uint32_t *count_dev, grt_stream_t stream) {
    if (!count_dev || (n && (!hits_dev || !indices_dev))) return GRT_ERR_INVALID_ARG;
    if (n > GRT_COMPACT_STATIC_MAX_HITS) return GRT_ERR_TOO_LARGE;
    uint32_t *tiles = nullptr;
    cudaError_t e = grt::static_tiles(&tiles);
    if (e == cudaSuccess) e = grt::launch_compact_hits(hits_dev, n, indices_dev, count_dev, tiles, (cudaStream_t)stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return GRT_ERR_CUDA;
    }
    return GRT_OK;
}
