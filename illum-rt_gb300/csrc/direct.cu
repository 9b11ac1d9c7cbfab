// Direct lighting kernels: the wavefront steps of the reference's direct-wf algorithm
// (k::sample_light, the shadow-ray trace, k::integrate_light; rt/cuda/bounce.cu:210-250,
// 380-410; or k::sample_uniform_dir / k::sample_cos_dir, the closest-hit trace,
// k::integrate_dir; bounce.cu:33-142, 341-375) and one fused persistent kernel doing all of them
// per pixel.
#include "direct.hpp"
#include "traverse.cuh"

namespace grt {

namespace {

constexpr unsigned kFull = 0xffffffffu;
using dl::f3;

// Materials beyond the table get the reference's default material (libgi/material.h:144-151).
__device__ __forceinline__ dl::material material_of(const dl_scene &ds, uint32_t id) {
    if (id < ds.n_mat) return ds.mats[id];
    dl::material m = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, 1.3f, 0.1f};
    return m;
}

__device__ __forceinline__ f3 vert(const dl_scene &ds, uint32_t i) {
    const float4 v = __ldg(ds.vpos + i);
    return {v.x, v.y, v.z};
}

// What the sampling step decides for one sample of one pixel.
struct dl_prep {
    bool emissive;  // the camera ray hit a light: its emission is added, no shadow ray
    f3 emis;
    f3 org, dir;
    float tmax;     // -FLT_MAX: no shadow ray
    f3 lcol;        // light sampling: the light's emission
    float pdf;
};

// k::sample_light (rt/cuda/bounce.cu:210-250), or k::sample_uniform_dir / k::sample_cos_dir
// (bounce.cu:33-142) for the direction strategies, for sample `s` of pixel `pixel`; random
// numbers from the PCG32 stream seed + s * n + pixel.
__device__ dl_prep prepare(const dl_scene &ds, f3 o, f3 d, float t, uint32_t ref, uint32_t pixel, uint32_t s,
                           uint32_t n, uint64_t seed, uint32_t sampling) {
    dl_prep p;
    p.emissive = false;
    p.emis = p.org = p.dir = p.lcol = {0.f, 0.f, 0.f};
    p.tmax = -FLT_MAX;
    p.pdf = 0.f;
    if (t == FLT_MAX) return p;
    const uint4 tri = __ldg(ds.tris + ref);
    const dl::material m = material_of(ds, tri.w);
    const f3 em = {m.emissive[0], m.emissive[1], m.emissive[2]};
    if (dl::not_black(em)) {
        p.emissive = true;
        p.emis = em;
        return p;
    }
    if (sampling != dl::kSampleLight) {
        pm::pcg32 rng;
        rng.set_sequence(seed + (uint64_t)s * n + pixel);
        const float x0 = rng.uniform(), x1 = rng.uniform();
        const f3 ns = pm::facing_normal(vert(ds, tri.x), vert(ds, tri.y), vert(ds, tri.z), d);
        p.org = {pm::add(o.x, pm::mul(t, d.x)), pm::add(o.y, pm::mul(t, d.y)), pm::add(o.z, pm::mul(t, d.z))};
        p.dir = dl::sample_dir(sampling, ns, x0, x1, p.pdf);
        p.tmax = FLT_MAX;
        return p;
    }
    if (ds.n_lights == 0) return p;
    pm::pcg32 rng;
    rng.set_sequence(seed + (uint64_t)s * n + pixel);
    const float x0 = rng.uniform(), x1 = rng.uniform(), x2 = rng.uniform();
    float pdf_l;
    const uint32_t id = dl::sample_light_index(ds.n_lights, ds.lf, ds.lcdf, ds.integral, x2, pdf_l);
    const uint4 L = __ldg(ds.lights + id);
    const dl::material lm = material_of(ds, L.w);
    const f3 from = {pm::add(o.x, pm::mul(t, d.x)), pm::add(o.y, pm::mul(t, d.y)), pm::add(o.z, pm::mul(t, d.z))};
    const dl::light_sample ls =
        dl::sample_li(from, vert(ds, L.x), vert(ds, L.y), vert(ds, L.z), {lm.emissive[0], lm.emissive[1], lm.emissive[2]},
                      x0, x1);
    p.lcol = ls.lcol;
    p.pdf = pm::mul(pdf_l, ls.pdf);
    if (dl::not_black(ls.lcol)) {
        p.org = ls.org;
        p.dir = ls.dir;
        p.tmax = ls.tmax;
    }
    return p;
}

// k::integrate_light (rt/cuda/bounce.cu:380-410): the radiance of one sample.
__device__ f3 radiance(const dl_scene &ds, f3 d, float t, uint32_t ref, f3 w_i, float tmax, f3 lcol, float pdf,
                       bool occluded) {
    if (t == FLT_MAX || !(tmax > 0.f) || occluded) return {0.f, 0.f, 0.f};
    const uint4 tri = __ldg(ds.tris + ref);
    const dl::material m = material_of(ds, tri.w);
    const f3 ns = pm::facing_normal(vert(ds, tri.x), vert(ds, tri.y), vert(ds, tri.z), d);
    return dl::integrate(lcol, {-d.x, -d.y, -d.z}, w_i, ns, m, pdf);
}

// k::integrate_dir (rt/cuda/bounce.cu:341-375): the radiance of one direction sample whose ray
// hit (sec_t, sec_ref): the emission of that triangle's material.
__device__ f3 radiance_dir(const dl_scene &ds, f3 d, float t, uint32_t ref, f3 w_i, float pdf, float sec_t,
                           uint32_t sec_ref) {
    if (t == FLT_MAX || sec_t == FLT_MAX) return {0.f, 0.f, 0.f};
    const uint4 tri = __ldg(ds.tris + ref);
    const dl::material m = material_of(ds, tri.w);
    const dl::material lm = material_of(ds, __ldg(ds.tris + sec_ref).w);
    const f3 ns = pm::facing_normal(vert(ds, tri.x), vert(ds, tri.y), vert(ds, tri.z), d);
    return dl::integrate({lm.emissive[0], lm.emissive[1], lm.emissive[2]}, {-d.x, -d.y, -d.z}, w_i, ns, m, pdf);
}

__device__ __forceinline__ float4 plus(float4 a, f3 b, float w) {
    return make_float4(pm::add(a.x, b.x), pm::add(a.y, b.y), pm::add(a.z, b.z), pm::add(a.w, w));
}

__device__ __forceinline__ ray_t shadow_ray(f3 o, f3 d, float tmax) {
    return make_ray(o.x, o.y, o.z, d.x, d.y, d.z, dl::kEps, tmax);  // the shadow ray's t_min (bounce.cu:246)
}

__global__ void __launch_bounds__(256) k_dl_sample(dl_scene ds, const float4 *__restrict__ rays,
                                                   const grt_hit *__restrict__ hits, uint32_t n, uint32_t s,
                                                   uint64_t seed, uint32_t sampling, float4 *shadow_rays,
                                                   float4 *lsample, float4 *fb) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 ro = rays[2 * (size_t)i], rd = rays[2 * (size_t)i + 1];
    const grt_hit h = hits[i];
    const dl_prep p = prepare(ds, {ro.x, ro.y, ro.z}, {rd.x, rd.y, rd.z}, h.t, h.ref, i, s, n, seed, sampling);
    if (p.emissive) fb[i] = plus(fb[i], p.emis, 0.f);
    shadow_rays[2 * (size_t)i] = make_float4(p.org.x, p.org.y, p.org.z, dl::kEps);
    shadow_rays[2 * (size_t)i + 1] = make_float4(p.dir.x, p.dir.y, p.dir.z, p.tmax);
    lsample[i] = make_float4(p.lcol.x, p.lcol.y, p.lcol.z, p.pdf);
}

__global__ void __launch_bounds__(256) k_dl_integrate(dl_scene ds, const float4 *__restrict__ rays,
                                                      const grt_hit *__restrict__ hits,
                                                      const float4 *__restrict__ shadow_rays,
                                                      const grt_hit *__restrict__ shadow_hits,
                                                      const float4 *__restrict__ lsample, uint32_t n,
                                                      uint32_t sampling, float4 *fb) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 rd = rays[2 * (size_t)i + 1];
    const grt_hit h = hits[i];
    const float4 sd = shadow_rays[2 * (size_t)i + 1];
    const float4 l = lsample[i];
    const grt_hit sh = shadow_hits[i];
    const f3 d = {rd.x, rd.y, rd.z}, w_i = {sd.x, sd.y, sd.z};
    const f3 rad = sampling == dl::kSampleLight
                       ? radiance(ds, d, h.t, h.ref, w_i, sd.w, {l.x, l.y, l.z}, l.w, sh.ref == 0xFFFFFFFFu)
                       : radiance_dir(ds, d, h.t, h.ref, w_i, l.w, sh.t, sh.ref);
    fb[i] = plus(fb[i], rad, 1.0f);
}

// add_hitpoint_albedo (rt/cuda/kernels.cu:170-197), untextured: fb += (albedo, 1) of the hit
// triangle's material, (0, 0, 0, 1) for a miss.
__device__ __forceinline__ float4 albedo_of(const dl_scene &ds, float t, uint32_t ref) {
    if (t == FLT_MAX) return make_float4(0.f, 0.f, 0.f, 1.f);
    const dl::material m = material_of(ds, __ldg(ds.tris + ref).w);
    return make_float4(m.albedo[0], m.albedo[1], m.albedo[2], 1.f);
}

__device__ __forceinline__ float4 plus4(float4 a, float4 b) {
    return make_float4(pm::add(a.x, b.x), pm::add(a.y, b.y), pm::add(a.z, b.z), pm::add(a.w, b.w));
}

__global__ void __launch_bounds__(256) k_add_albedo(dl_scene ds, const grt_hit *__restrict__ hits, uint32_t n,
                                                    float4 *fb) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const grt_hit h = hits[i];
    fb[i] = plus4(fb[i], albedo_of(ds, h.t, h.ref));
}

// Fused form, warp-synchronous: a warp takes 32 consecutive pixels from the global counter,
// traverses their camera rays together (closest hit), then for each sample prepares the
// samples, traverses their rays together (any hit for shadow rays to a light, closest hit for
// sampled directions) and integrates into registers, in the order the wavefront steps add to
// the frame buffer. All lanes of a warp are always in the same phase, so every loop order works,
// the speculative ones included, and the rays of one sample stay as coherent as in the
// wavefront form.
template <int ORDER, bool ANY>
__device__ __forceinline__ void trace_all(trav_t &s, bool active, bool plain, const dev_scene &sc, const ray_t &r,
                                          int *stk, int stride, int cap, unsigned *err) {
    constexpr bool SPEC = ORDER == SPECULATIVE || ORDER == WIDE_SPECULATIVE;
    constexpr bool WIDE = ORDER == WIDE_SPECULATIVE;
    while (__any_sync(kFull, active && !s.done)) {
        if (SPEC && __all_sync(kFull, !active || plain))
            trav_spec_iter<ANY, false, WIDE, false, kSpecDirect.visits, kSpecDirect.pend, true>(
                s, active, plain, sc, r, stk, stride, cap,
                spec_cfg{kSpecDirect.pend, kSpecDirect.exit, kSpecDirect.visits}, err);
        else if (SPEC)
            trav_spec_iter<ANY, false, WIDE, false, kSpecDirect.visits, kSpecDirect.pend>(s, active, plain, sc, r, stk,
                                                                                           stride, cap,
                                                   spec_cfg{kSpecDirect.pend, kSpecDirect.exit, kSpecDirect.visits},
                                                   err);
        else if (active && !s.done && plain)
            trav_advance<ORDER, ANY, false, true>(s, sc, r, stk, stride, cap, err);
        else if (active && !s.done)
            trav_advance<ORDER, ANY, false, false>(s, sc, r, stk, stride, cap, err);
    }
}

// DIR: a direction strategy (closest-hit rays, k::integrate_dir) instead of light sampling
// (any-hit shadow rays, k::integrate_light).
template <int ORDER, bool DIR>
__global__ void __launch_bounds__(256) k_dl_fused(dev_scene sc, dl_scene ds, const float4 *__restrict__ rays,
                                                  uint32_t n, uint32_t samples, uint64_t seed, uint32_t sampling,
                                                  uint32_t albedo, float4 *fb, unsigned *err, unsigned *counter,
                                                  int cap) {
    extern __shared__ int s_stack[];
    if (stop_requested_at_entry(err)) return;  // the host asked the context to stop
    constexpr bool WIDE = ORDER == WIDE_SPECULATIVE;
    const unsigned lane = threadIdx.x & 31u;
    int *stk = s_stack + threadIdx.x;
    const int stride = blockDim.x;
    for (;;) {
        unsigned base = 0;
        if (lane == 0) base = atomicAdd(counter, 32u);
        base = __shfl_sync(kFull, base, 0);
        if (base >= n) break;
        const uint32_t pix = base + lane;
        const bool active = pix < n;
        ray_t r = {};
        trav_t s;
        if (active) r = load_ray(rays, pix);
        const f3 o = {r.ox(), r.oy(), r.oz()}, d = {r.dx, r.dy, r.dz};
        float4 acc = active ? fb[pix] : make_float4(0.f, 0.f, 0.f, 0.f);
        trav_init(s, sc, r, WIDE);
        bool plain = active && sc.finite && ray_is_plain(r);
        trace_all<ORDER, false>(s, active, plain, sc, r, stk, stride, cap, err);
        const float ht = active ? s.hit.t : FLT_MAX;
        const uint32_t href = s.hit.ref;
        if (albedo && active) acc = plus4(acc, albedo_of(ds, ht, href));  // primary-wf's shading
        for (uint32_t smp = 0; smp < samples; ++smp) {
            dl_prep p;
            if (active) {
                p = prepare(ds, o, d, ht, href, pix, smp, n, seed, DIR ? sampling : dl::kSampleLight);
                if (p.emissive) acc = plus(acc, p.emis, 0.f);
            }
            const bool shoot = active && p.tmax > 0.f;  // a ray that can find an occluder / a light
            if (shoot) r = shadow_ray(p.org, p.dir, p.tmax);
            trav_init(s, sc, r, WIDE);
            plain = shoot && sc.finite && ray_is_plain(r);
            trace_all<ORDER, !DIR>(s, shoot, plain, sc, r, stk, stride, cap, err);
            if (active) {
                f3 rad = {0.f, 0.f, 0.f};
                if (shoot)
                    rad = DIR ? radiance_dir(ds, d, ht, href, p.dir, p.pdf, s.hit.t, s.hit.ref)
                              : radiance(ds, d, ht, href, p.dir, p.tmax, p.lcol, p.pdf, s.found);
                acc = plus(acc, rad, 1.0f);
            }
        }
        if (active) fb[pix] = acc;
    }
}

template <int ORDER, bool DIR> const void *fused_ptr() { return (const void *)k_dl_fused<ORDER, DIR>; }

template <int ORDER, bool DIR>
cudaError_t fused_run(const dev_scene &sc, const dl_scene &ds, const float4 *rays, uint32_t n, uint32_t samples,
                      uint64_t seed, uint32_t sampling, uint32_t albedo, float4 *fb, int stack_entries, int bt,
                      int num_sms, unsigned *err, unsigned *counter, cudaStream_t st) {
    const size_t smem = (size_t)stack_entries * bt * sizeof(int);
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_dl_fused<ORDER, DIR>, bt, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    e = cudaMemsetAsync(counter, 0, sizeof(unsigned), st);
    if (e != cudaSuccess) return e;
    k_dl_fused<ORDER, DIR><<<per_sm * num_sms, bt, smem, st>>>(sc, ds, rays, n, samples, seed, sampling, albedo, fb,
                                                                err, counter, stack_entries);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_dl_sample(const dl_scene &ds, const float4 *rays, const grt_hit *hits, uint32_t n, uint32_t s,
                             uint64_t seed, uint32_t sampling, float4 *shadow_rays, float4 *lsample, float4 *fb,
                             cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    k_dl_sample<<<(n + 255) / 256, 256, 0, st>>>(ds, rays, hits, n, s, seed, sampling, shadow_rays, lsample, fb);
    return cudaGetLastError();
}

cudaError_t launch_dl_integrate(const dl_scene &ds, const float4 *rays, const grt_hit *hits, const float4 *shadow_rays,
                                const grt_hit *shadow_hits, const float4 *lsample, uint32_t n, uint32_t sampling,
                                float4 *fb, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    k_dl_integrate<<<(n + 255) / 256, 256, 0, st>>>(ds, rays, hits, shadow_rays, shadow_hits, lsample, n, sampling,
                                                    fb);
    return cudaGetLastError();
}

cudaError_t launch_add_albedo(const dl_scene &ds, const grt_hit *hits, uint32_t n, float4 *fb, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    k_add_albedo<<<(n + 255) / 256, 256, 0, st>>>(ds, hits, n, fb);
    return cudaGetLastError();
}

cudaError_t launch_dl_fused(const dev_scene &sc, const dl_scene &ds, const float4 *rays, uint32_t n, uint32_t samples,
                            uint64_t seed, uint32_t sampling, uint32_t albedo, float4 *fb, int order,
                            int stack_entries, int bt, int num_sms, unsigned *err, unsigned *counter,
                            cudaStream_t st) {
    if (n == 0) return cudaSuccess;
#define GRT_DL_RUN(O)                                                                                             \
    return sampling == dl::kSampleLight                                                                          \
               ? fused_run<O, false>(sc, ds, rays, n, samples, seed, sampling, albedo, fb, stack_entries, bt,     \
                                     num_sms, err, counter, st)                                                   \
               : fused_run<O, true>(sc, ds, rays, n, samples, seed, sampling, albedo, fb, stack_entries, bt,      \
                                    num_sms, err, counter, st)
    switch (order) {
        case IF_IF: GRT_DL_RUN(IF_IF);
        case SPECULATIVE: GRT_DL_RUN(SPECULATIVE);
        case WIDE_SPECULATIVE: GRT_DL_RUN(WIDE_SPECULATIVE);
        default: GRT_DL_RUN(WHILE_WHILE);
    }
#undef GRT_DL_RUN
}

cudaError_t prepare_dl_kernels() {
    const int bytes = kStackLarge * 256 * (int)sizeof(int);
    for (const void *f : {fused_ptr<IF_IF, false>(), fused_ptr<WHILE_WHILE, false>(), fused_ptr<SPECULATIVE, false>(),
                          fused_ptr<WIDE_SPECULATIVE, false>(), fused_ptr<IF_IF, true>(), fused_ptr<WHILE_WHILE, true>(),
                          fused_ptr<SPECULATIVE, true>(), fused_ptr<WIDE_SPECULATIVE, true>()}) {
        cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

}  // namespace grt
