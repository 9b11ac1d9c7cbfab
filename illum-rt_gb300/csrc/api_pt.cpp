// C-ABI of the ray-generation steps around the traversal (compaction, shadow rays) and of the
// diffuse path tracer (include/grt.h), including capture and replay of the path-tracing step as
// a CUDA graph.
//
// All of them take their temporary buffers from one scratch arena per context, grown on
// demand; calls that use it must be ordered on one stream (a context is not thread-safe).
#include <cstring>

#include "ctx.hpp"
#include "adjoint.hpp"
#include "pathtrace.hpp"

using namespace grt;

namespace {

inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

grt_status ensure_scratch(grt_ctx *c, size_t bytes) {
    if (c->scratch_bytes >= bytes) return GRT_OK;
    if (c->d_scratch) cudaFree(c->d_scratch);
    c->d_scratch = nullptr;
    c->scratch_bytes = 0;
    cudaError_t e = cudaMalloc(&c->d_scratch, bytes);
    if (e != cudaSuccess) return cuda_fail(c, e, "allocating scratch memory");
    c->scratch_bytes = bytes;
    return GRT_OK;
}

pt_scene scene_for_shading(grt_ctx *c) {
    return {(const float4 *)c->d_vpos, (const uint4 *)c->d_tris, c->d_albedo, c->n_albedo};
}

// Carves the arena: [hit list | compaction counts | counters (64 words) | wavefront buffers].
struct pt_layout {
    size_t hit_list, compact, counters, states, queue0, queue1, rays0, rays1, hits, starts, total;
};

pt_layout layout_for(uint32_t n_primary, uint32_t n_paths, bool wavefront) {
    pt_layout L{};
    size_t off = 0;
    L.hit_list = off;
    off = align256(off + (size_t)n_primary * 4);
    L.compact = off;
    off = align256(off + compact_scratch_bytes(n_primary));
    L.counters = off;
    off = align256(off + 64 * 4);
    if (wavefront) {
        L.states = off;
        off = align256(off + (size_t)n_paths * wavefront_state_bytes());
        L.queue0 = off;
        off = align256(off + (size_t)n_paths * 4);
        L.queue1 = off;
        off = align256(off + (size_t)n_paths * 4);
        L.rays0 = off;
        off = align256(off + (size_t)n_paths * 32);
        L.rays1 = off;
        off = align256(off + (size_t)n_paths * 32);
        L.hits = off;
        off = align256(off + (size_t)n_paths * 16);
    } else {
        L.starts = off;
        off = align256(off + (size_t)n_paths * 32);
    }
    L.total = off;
    return L;
}

template <typename T> T *at(grt_ctx *c, size_t off) { return (T *)((char *)c->d_scratch + off); }

// Enqueues one path-tracing step on `st` (no allocation, no synchronisation: capturable).
cudaError_t enqueue_pathtrace(grt_ctx *c, const grt_pt_params &p, const pt_params_dev &pp, const launch_params &lp,
                              const launch_params &lp_trace, const pt_layout &L, const float *prim_rays,
                              const grt_hit *prim_hits, uint32_t n_primary, uint32_t n_paths,
                              grt_path_result *results, grt_hit *bounce_hits, cudaStream_t st) {
    const pt_scene ps = scene_for_shading(c);
    uint32_t *hit_list = at<uint32_t>(c, L.hit_list);
    uint32_t *counters = at<uint32_t>(c, L.counters);
    uint32_t *n_list = counters;  // [0] valid primary hits, [1..] queue sizes
    cudaError_t e = cudaMemsetAsync(counters, 0, 64 * 4, st);
    if (e == cudaSuccess)
        e = launch_compact_hits(prim_hits, n_primary, hit_list, n_list, at<uint32_t>(c, L.compact), st);
    if (e != cudaSuccess) return e;
    if (p.mode == GRT_PT_FUSED)
        return launch_fused(scene_for(c), ps, pp, (const float4 *)prim_rays, prim_hits, n_primary, hit_list, n_list,
                            n_paths, results, bounce_hits, lp, c->d_err, c->d_counter, at<float4>(c, L.starts), st);
    uint32_t *queue[2] = {at<uint32_t>(c, L.queue0), at<uint32_t>(c, L.queue1)};
    float4 *rays[2] = {at<float4>(c, L.rays0), at<float4>(c, L.rays1)};
    grt_hit *hits = at<grt_hit>(c, L.hits);
    void *states = at<void>(c, L.states);
    e = launch_wavefront_init(ps, pp, (const float4 *)prim_rays, prim_hits, hit_list, n_list, n_paths, states, queue[0],
                              rays[0], results, counters + 1, st);
    for (uint32_t b = 1; b <= p.max_bounces && e == cudaSuccess; ++b) {
        const int cur = (b - 1) & 1, nxt = b & 1;
        e = launch_trace_plain(scene_for(c), rays[cur], hits, n_paths, false, lp_trace, c->d_err, st, counters + b);
        if (e == cudaSuccess)
            e = launch_wavefront_shade(ps, pp, n_paths, counters + b, queue[cur], rays[cur], hits, states,
                                       counters + b + 1, queue[nxt], rays[nxt], results, bounce_hits, st);
    }
    return e;
}

uint64_t fbits(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
}

}  // namespace

extern "C" {

void grt_pt_params_default(grt_pt_params *p) {
    if (!p) return;
    p->max_bounces = 5;
    p->rr_start = 3;
    p->rr_continue = 0.8f;
    p->eps = 1e-4f;
    p->seed = 0;
    p->mode = GRT_PT_FUSED;
    p->use_graph = 0;
}

grt_status grt_set_materials(grt_ctx *c, const float *albedo, uint32_t n) {
    return guarded(c, [&]() -> grt_status {
        if (!c || (n && !albedo)) return GRT_ERR_INVALID_ARG;
        device_guard g(c->device);
        if (c->d_albedo) cudaFree(c->d_albedo);
        c->d_albedo = nullptr;
        c->n_albedo = 0;
        if (n == 0) return GRT_OK;
        cudaError_t e = cudaMalloc(&c->d_albedo, (size_t)n * 4);
        if (e == cudaSuccess) e = cudaMemcpy(c->d_albedo, albedo, (size_t)n * 4, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return cuda_fail(c, e, "uploading materials");
        c->n_albedo = n;
        return GRT_OK;
    });
}

grt_status grt_compact_hits(grt_ctx *c, const grt_hit *hits_dev, uint32_t n, uint32_t *indices_dev,
                            uint32_t *count_dev, grt_stream_t stream) {
    return guarded(c, [&]() -> grt_status {
        if (!c) return GRT_ERR_INVALID_ARG;
        if (!count_dev || (n && (!hits_dev || !indices_dev)))
            return fail(c, GRT_ERR_INVALID_ARG, "null buffer for grt_compact_hits");
        device_guard g(c->device);
        timed_call timer(c, GRT_TIME_RAYS, (cudaStream_t)stream);
        grt_status s = ensure_scratch(c, compact_scratch_bytes(n));
        if (s != GRT_OK) return s;
        cudaError_t e = launch_compact_hits(hits_dev, n, indices_dev, count_dev, (uint32_t *)c->d_scratch,
                                            (cudaStream_t)stream);
        return e == cudaSuccess ? GRT_OK : cuda_fail(c, e, "launching the compaction");
    });
}

grt_status grt_shadow_rays(grt_ctx *c, const float *rays_dev, const grt_hit *hits_dev, uint32_t n,
                           const float light[3], float eps, float *shadow_rays_dev, uint32_t *count_dev,
                           grt_stream_t stream) {
    return guarded(c, [&]() -> grt_status {
        if (!c) return GRT_ERR_INVALID_ARG;
        if (!c->built) return fail(c, GRT_ERR_NOT_BUILT, "grt_shadow_rays before a successful grt_build");
        if (!light || !count_dev || (n && (!rays_dev || !hits_dev || !shadow_rays_dev)) || !aligned16(rays_dev) ||
            !aligned16(shadow_rays_dev) || !aligned16(hits_dev))
            return fail(c, GRT_ERR_INVALID_ARG, "null or misaligned buffer for grt_shadow_rays");
        device_guard g(c->device);
        timed_call timer(c, GRT_TIME_RAYS, (cudaStream_t)stream);
        grt_status s = ensure_scratch(c, compact_scratch_bytes(n));
        if (s != GRT_OK) return s;
        cudaError_t e = launch_shadow_rays(scene_for_shading(c), (const float4 *)rays_dev, hits_dev, n, light, eps,
                                           (float4 *)shadow_rays_dev, count_dev, (uint32_t *)c->d_scratch,
                                           (cudaStream_t)stream);
        return e == cudaSuccess ? GRT_OK : cuda_fail(c, e, "launching the shadow-ray setup");
    });
}

grt_status grt_pathtrace(grt_ctx *c, const grt_pt_params *params, const float *prim_rays_dev,
                         const grt_hit *prim_hits_dev, uint32_t n_primary, uint32_t n_paths,
                         grt_path_result *results_dev, grt_hit *bounce_hits_dev, grt_stream_t stream) {
    return guarded(c, [&]() -> grt_status {
        if (!c) return GRT_ERR_INVALID_ARG;
        if (!c->built) return fail(c, GRT_ERR_NOT_BUILT, "grt_pathtrace before a successful grt_build");
        grt_pt_params p;
        grt_pt_params_default(&p);
        if (params) p = *params;
        if (n_paths == 0) return GRT_OK;
        if (n_primary == 0 || !prim_rays_dev || !prim_hits_dev || !results_dev || !aligned16(prim_rays_dev) ||
            !aligned16(prim_hits_dev) || !aligned16(results_dev) || !aligned16(bounce_hits_dev))
            return fail(c, GRT_ERR_INVALID_ARG, "null or misaligned buffer for grt_pathtrace");
        if (p.max_bounces < 1 || p.max_bounces > 60 || !(p.rr_continue > 0.f && p.rr_continue <= 1.f) ||
            (p.mode != GRT_PT_WAVEFRONT && p.mode != GRT_PT_FUSED) || n_paths > (1u << 31) || n_primary > (1u << 31))
            return fail(c, GRT_ERR_INVALID_ARG, "invalid path-tracing parameters");
        if (p.use_graph && !stream)
            return fail(c, GRT_ERR_INVALID_ARG, "graph replay needs a stream other than the legacy default stream");
        if (needed_stack(c) > grt::kStackLarge)
            return fail(c, GRT_ERR_BVH_TOO_DEEP, "the selected tracer needs a deeper stack than the kernels have");
        device_guard g(c->device);
        timed_call timer(c, GRT_TIME_PATHTRACE, (cudaStream_t)stream);
        const bool wavefront = p.mode == GRT_PT_WAVEFRONT;
        const pt_layout L = layout_for(n_primary, n_paths, wavefront);
        grt_status s = ensure_scratch(c, L.total);
        if (s != GRT_OK) return s;
        const pt_params_dev pp = {p.max_bounces, p.rr_start, p.rr_continue, p.eps, p.seed};
        launch_params lp_trace = params_for(c, false);  // one-thread-per-ray kernel of the wavefront form
        launch_params lp = lp_trace;
        lp.spec = tuned_spec(c->tuning, kSpecPaths);
        lp.grid_blocks = (c->tuning.blocks_per_sm > 0 ? c->tuning.blocks_per_sm
                                                      : fused_blocks_per_sm(lp.block_threads, lp.stack_entries, lp.order, scene_for(c).alpha != nullptr,
                                                                          lp.spec)) *
                         c->num_sms;
        cudaStream_t st = (cudaStream_t)stream;
        if (!p.use_graph) {
            cudaError_t e = enqueue_pathtrace(c, p, pp, lp, lp_trace, L, prim_rays_dev, prim_hits_dev, n_primary, n_paths,
                                              results_dev, bounce_hits_dev, st);
            return e == cudaSuccess ? GRT_OK : cuda_fail(c, e, "launching the path tracer");
        }
        const std::vector<uint64_t> key = {
            (uint64_t)p.mode, (uint64_t)(uintptr_t)prim_rays_dev, (uint64_t)(uintptr_t)prim_hits_dev, n_primary,
            n_paths, (uint64_t)(uintptr_t)results_dev, (uint64_t)(uintptr_t)bounce_hits_dev, p.max_bounces, p.rr_start,
            fbits(p.rr_continue), fbits(p.eps), p.seed, (uint64_t)(uintptr_t)c->d_scratch, c->scene_generation,
            (uint64_t)(uintptr_t)c->d_albedo, c->n_albedo, (uint64_t)(uintptr_t)st, (uint64_t)lp.block_threads,
            (uint64_t)lp.grid_blocks, (uint64_t)lp.refill_threshold, (uint64_t)lp.refill_period,
            (uint64_t)lp.stack_entries, (uint64_t)lp.order, (uint64_t)lp_trace.block_threads, (uint64_t)lp.spec.pend,
            (uint64_t)lp.spec.exit, (uint64_t)lp.spec.visits,
            (uint64_t)(uintptr_t)lp_trace.counters, (uint64_t)(uintptr_t)scene_for(c).alpha};
        if (!c->pt_graph.exec || c->pt_graph.key != key) {
            if (c->pt_graph.exec) cudaGraphExecDestroy(c->pt_graph.exec);
            c->pt_graph.exec = nullptr;
            cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
            if (e != cudaSuccess) return cuda_fail(c, e, "beginning the graph capture");
            cudaError_t el = enqueue_pathtrace(c, p, pp, lp, lp_trace, L, prim_rays_dev, prim_hits_dev, n_primary,
                                               n_paths, results_dev, bounce_hits_dev, st);
            cudaGraph_t graph = nullptr;
            e = cudaStreamEndCapture(st, &graph);
            if (el != cudaSuccess || e != cudaSuccess) {
                if (graph) cudaGraphDestroy(graph);
                return cuda_fail(c, el != cudaSuccess ? el : e, "capturing the path-tracing step");
            }
            e = cudaGraphInstantiate(&c->pt_graph.exec, graph, 0);
            cudaGraphDestroy(graph);
            if (e != cudaSuccess) {
                c->pt_graph.exec = nullptr;
                return cuda_fail(c, e, "instantiating the path-tracing graph");
            }
            c->pt_graph.key = key;
        }
        cudaError_t e = cudaGraphLaunch(c->pt_graph.exec, st);
        return e == cudaSuccess ? GRT_OK : cuda_fail(c, e, "launching the path-tracing graph");
    });
}

grt_status grt_adjoint(grt_ctx *c, const float *rays_dev, const grt_hit *hits_dev, const float *grad_hits_dev,
                       uint32_t n, const float *vpos_dev, uint32_t vstride, float *grad_vpos_dev, float *grad_rays_dev,
                       grt_stream_t stream) {
    return guarded(c, [&]() -> grt_status {
        if (!c) return GRT_ERR_INVALID_ARG;
        if (!c->built) return fail(c, GRT_ERR_NOT_BUILT, "grt_adjoint before a successful grt_build");
        if (n == 0) return GRT_OK;
        if (!rays_dev || !hits_dev || !grad_hits_dev || !aligned16(rays_dev) || !aligned16(hits_dev) ||
            !aligned16(grad_rays_dev) || (vpos_dev && vstride != 3 && vstride != 4))
            return fail(c, GRT_ERR_INVALID_ARG, "invalid buffer or vertex stride for grt_adjoint");
        device_guard g(c->device);
        timed_call timer(c, GRT_TIME_ADJOINT, (cudaStream_t)stream);
        const float4 *vp = vpos_dev ? (const float4 *)vpos_dev : (const float4 *)c->d_vpos;
        const uint32_t stride = vpos_dev ? vstride : 4;
        cudaError_t e = launch_adjoint((const float4 *)rays_dev, hits_dev, grad_hits_dev, n, vp, stride,
                                       (const uint4 *)c->d_tris, grad_vpos_dev, (float4 *)grad_rays_dev,
                                       (cudaStream_t)stream);
        return e == cudaSuccess ? GRT_OK : cuda_fail(c, e, "launching the adjoint kernel");
    });
}

}  // extern "C"
