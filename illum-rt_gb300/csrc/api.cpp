// C-ABI of libgrt.so (include/grt.h): context, BVH build/upload, tracer selection, launches.
//
// This is the GB300 counterpart of wf::cuda::batch_rt (rt/cuda/base.h:403-429) and of the
// CUDA platform's tracer registry (rt/cuda/platform.cpp:34-56, 102-131), reduced to plain
// pointers, sizes and status codes.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "ctx.hpp"
#include "direct.hpp"
#include "multi.hpp"
#include "pathtrace.hpp"

using namespace grt;

extern "C" {

int grt_version(void) { return GRT_VERSION_MAJOR * 1000 + GRT_VERSION_MINOR; }

void grt_bvh_opts_default(grt_bvh_opts *o) {
    if (!o) return;
    o->split = GRT_SPLIT_SAH;
    o->max_tris_per_node = 4;
    o->number_of_planes = 16;
    o->esc = 1;
}

grt_status grt_create(const grt_config *cfg, grt_ctx **out) {
    return guarded(nullptr, [&]() -> grt_status {
        if (!out) return GRT_ERR_INVALID_ARG;
        *out = nullptr;
        int dev = cfg ? cfg->device : 0;
        int count = 0;
        if (cudaGetDeviceCount(&count) != cudaSuccess || dev < 0 || dev >= count) {
            cudaGetLastError();
            return GRT_ERR_NO_DEVICE;
        }
        grt_ctx *c = new grt_ctx();
        c->device = dev;
        device_guard g(dev);
        cudaError_t e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess) e = cudaMalloc(&c->d_err, grt::kStatusWords * sizeof(unsigned));
        if (e == cudaSuccess) {
            c->d_counter = c->d_err + grt::kStatusCounter;
            e = cudaMemset(c->d_err, 0, grt::kStatusWords * sizeof(unsigned));
        }
        if (e == cudaSuccess) e = cudaHostAlloc((void **)&c->h_flag, 3 * sizeof(unsigned), cudaHostAllocDefault);
        if (e == cudaSuccess) {
            c->h_flag[0] = 1u;
            c->h_flag[1] = 0u;
            c->h_flag[2] = grt::kAbortCounter;
            e = cudaStreamCreateWithFlags(&c->abort_stream, cudaStreamNonBlocking);
        }
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = grt::prepare_trace_kernels();
        if (e == cudaSuccess) e = grt::prepare_pt_kernels();
        if (e == cudaSuccess) e = grt::prepare_multi_kernels();
        if (e == cudaSuccess) e = grt::prepare_dl_kernels();
        if (e != cudaSuccess) {
            cudaGetLastError();
            if (c->d_err) cudaFree(c->d_err);
            if (c->h_flag) cudaFreeHost(c->h_flag);
            if (c->abort_stream) cudaStreamDestroy(c->abort_stream);
            delete c;
            return e == cudaErrorMemoryAllocation ? GRT_ERR_OOM : GRT_ERR_CUDA;
        }
        *out = c;
        return GRT_OK;
    });
}

grt_status grt_destroy(grt_ctx *c) {
    if (!c) return GRT_ERR_INVALID_ARG;
    {
        device_guard g(c->device);
        free_scene(c);
        grt_free_multi(c);
        if (c->d_stage) cudaFree(c->d_stage);
        if (c->d_scratch) cudaFree(c->d_scratch);
        if (c->d_albedo) cudaFree(c->d_albedo);
        if (c->d_dl_scratch) cudaFree(c->d_dl_scratch);
        if (c->d_extent) cudaFree(c->d_extent);
        for (const auto &q : c->timing.pending) {
            cudaEventDestroy(q.a);
            cudaEventDestroy(q.b);
        }
        for (cudaEvent_t e : c->timing.pool) cudaEventDestroy(e);
        if (c->pt_graph.exec) cudaGraphExecDestroy(c->pt_graph.exec);
        if (c->d_err) cudaFree(c->d_err);
        if (c->h_flag) cudaFreeHost(c->h_flag);
        if (c->abort_stream) cudaStreamDestroy(c->abort_stream);
        if (c->stream) cudaStreamDestroy(c->stream);
    }
    delete c;
    return GRT_OK;
}

const char *grt_last_error(const grt_ctx *c) { return c ? c->err.c_str() : "null context"; }

grt_status grt_build(grt_ctx *c, const float *vpos4, uint32_t nv, const uint32_t *tris4, uint32_t nt,
                     const grt_bvh_opts *opts) {
    return guarded(c, [&]() -> grt_status {
        if (!c) return GRT_ERR_INVALID_ARG;
        if ((nv && !vpos4) || (nt && !tris4)) return fail(c, GRT_ERR_INVALID_ARG, "null vertex or triangle array");
        const grt::build_opts bo = to_build_opts(opts);
        device_guard g(c->device);
        free_scene(c);
        ++c->scene_generation;
        c->stats = grt_bvh_stats{};

        auto t0 = std::chrono::steady_clock::now();
        std::string msg;
        grt::ref_tree tree;
        if (!grt::build_or_load(c, vpos4, nv, tris4, nt, bo, tree, msg)) return fail(c, GRT_ERR_INVALID_ARG, msg);
        c->stats.build_ms = ms_since(t0);

        t0 = std::chrono::steady_clock::now();
        grt::flat_bvh flat;
        if (!grt::flatten_bvh(tree, vpos4, tris4, flat, msg)) return fail(c, GRT_ERR_INVALID_ARG, msg);
        c->stats.flatten_ms = ms_since(t0);
        grt::flat_bvh4 wide;
        if (!grt::flatten_bvh4(tree, flat, wide, msg)) return fail(c, GRT_ERR_INVALID_ARG, msg);
        c->stats.flatten_ms = ms_since(t0);
        if (flat.depth > (uint32_t)grt::kStackLarge)
            return fail(c, GRT_ERR_BVH_TOO_DEEP,
                        "BVH depth " + std::to_string(flat.depth) + " exceeds the largest traversal stack (" +
                            std::to_string(grt::kStackLarge) + ")");
        bool finite = true;
        for (size_t i = 0; i < (size_t)nv && finite; ++i)
            for (int k = 0; k < 3; ++k) finite = finite && std::isfinite(vpos4[4 * i + k]);

        t0 = std::chrono::steady_clock::now();
        const size_t nb = flat.nodes.size() * 4, rb = flat.records.size() * 4;
        const size_t vb = (size_t)nv * 16, tb = (size_t)nt * 16;
        cudaError_t e = cudaSuccess;
        auto up = [&](void **dst, const void *src, size_t bytes) {
            if (e != cudaSuccess || bytes == 0) return;
            e = cudaMalloc(dst, bytes);
            if (e == cudaSuccess) e = cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice);
        };
        up(&c->d_nodes, flat.nodes.data(), nb);
        up(&c->d_nodes4, wide.nodes.data(), wide.nodes.size() * 4);
        up(&c->d_recs, flat.records.data(), rb);
        up(&c->d_vpos, vpos4, vb);
        up(&c->d_tris, tris4, tb);
        up(&c->d_parent, flat.parent.data(), flat.parent.size() * 4);
        up(&c->d_wide_index, wide.wide_index.data(), wide.wide_index.size() * 4);
        if (e != cudaSuccess) {
            free_scene(c);
            return cuda_fail(c, e, "uploading the BVH");
        }
        c->n_links = flat.inner;
        c->n_records = (uint32_t)(flat.records.size() / 12);
        c->stats.upload_ms = ms_since(t0);

        c->sc.nodes = (const float4 *)c->d_nodes;
        c->sc.records = (const float4 *)c->d_recs;
        c->sc.root = flat.root;
        c->sc.nodes4 = (const float4 *)c->d_nodes4;
        c->sc.root4 = wide.root;
        c->stack_bound4 = wide.stack_bound;
        c->sc.empty = flat.empty ? 1 : 0;
        c->sc.finite = finite ? 1 : 0;
        c->nv = nv;
        c->nt = nt;
        c->depth = flat.depth;
        c->stats.ref_nodes = (uint32_t)tree.nodes.size();
        c->stats.inner_nodes = flat.inner;
        c->stats.tri_records = (uint32_t)tree.index.size();
        c->stats.depth = flat.depth;
        c->stats.device_bytes = nb + rb + vb + tb + wide.nodes.size() * 4;
        c->tree = std::move(tree);
        c->built = true;
        return GRT_OK;
    });
}

grt_status grt_set_alpha(grt_ctx *c, const float *tc2, uint32_t nv, const int32_t *mat_tex, uint32_t n_mat,
                         const grt_alpha_texture *tex, uint32_t n_tex) {
    return guarded(c, [&]() -> grt_status {
        if (!c) return GRT_ERR_INVALID_ARG;
        device_guard g(c->device);
        if (c->d_alpha) cudaFree(c->d_alpha);
        c->d_alpha = nullptr;
        ++c->scene_generation;  // captured path-tracing graphs hold the old scene
        if (!mat_tex) return GRT_OK;
        if (!c->built) return fail(c, GRT_ERR_NOT_BUILT, "grt_set_alpha before a successful build");
        if (nv != c->nv || (nv && !tc2) || (n_tex && !tex))
            return fail(c, GRT_ERR_INVALID_ARG, "texture coordinates must cover the built scene's vertices");
        size_t texels = 0;
        for (uint32_t k = 0; k < n_tex; ++k) {
            if (!tex[k].alpha || tex[k].width == 0 || tex[k].height == 0 || tex[k].width > (1u << 24) ||
                tex[k].height > (1u << 24))
                return fail(c, GRT_ERR_INVALID_ARG, "texture " + std::to_string(k) + ": empty or oversized");
            texels += (size_t)tex[k].width * tex[k].height;
        }
        if (texels >= (1ull << 32)) return fail(c, GRT_ERR_INVALID_ARG, "more than 2^32 texels");
        for (uint32_t m = 0; m < n_mat; ++m)
            if (mat_tex[m] < -1 || mat_tex[m] >= (int32_t)n_tex)
                return fail(c, GRT_ERR_INVALID_ARG, "material " + std::to_string(m) + " names no texture");
        // one allocation: descriptor, texture coordinates, material table, texture table, texels
        auto a16 = [](size_t b) { return (b + 15) & ~(size_t)15; };
        const size_t o_tc = a16(sizeof(alpha_data)), o_mat = o_tc + a16((size_t)nv * 8),
                     o_tex = o_mat + a16((size_t)n_mat * 4), o_texels = o_tex + a16((size_t)n_tex * 16),
                     total = o_texels + std::max<size_t>(texels * 4, 4);
        std::vector<char> host(total, 0);
        std::vector<uint4> table(n_tex);
        size_t first = 0;
        for (uint32_t k = 0; k < n_tex; ++k) {
            table[k] = make_uint4(tex[k].width, tex[k].height, (uint32_t)first, 0u);
            std::memcpy(host.data() + o_texels + first * 4, tex[k].alpha, (size_t)tex[k].width * tex[k].height * 4);
            first += (size_t)tex[k].width * tex[k].height;
        }
        if (nv) std::memcpy(host.data() + o_tc, tc2, (size_t)nv * 8);
        if (n_mat) std::memcpy(host.data() + o_mat, mat_tex, (size_t)n_mat * 4);
        if (n_tex) std::memcpy(host.data() + o_tex, table.data(), (size_t)n_tex * 16);
        char *dev = nullptr;
        cudaError_t e = cudaMalloc(&dev, total);
        if (e != cudaSuccess) return cuda_fail(c, e, "allocating the texture data");
        alpha_data d;
        d.tris = (const uint4 *)c->d_tris;
        d.tc = (const float2 *)(dev + o_tc);
        d.mat_tex = (const int32_t *)(dev + o_mat);
        d.tex = (const uint4 *)(dev + o_tex);
        d.texels = (const float *)(dev + o_texels);
        d.n_mat = n_mat;
        std::memcpy(host.data(), &d, sizeof(d));
        e = cudaMemcpy(dev, host.data(), total, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            cudaFree(dev);
            return cuda_fail(c, e, "uploading the texture data");
        }
        c->d_alpha = dev;
        return GRT_OK;
    });
}

grt_status grt_bvh_info(grt_ctx *c, grt_bvh_stats *out) {
    if (!c || !out) return GRT_ERR_INVALID_ARG;
    if (!c->built) return fail(c, GRT_ERR_NOT_BUILT, "no scene has been built");
    *out = c->stats;
    return GRT_OK;
}

grt_status grt_export_bvh(grt_ctx *c, uint32_t *nodes14, uint32_t *index, uint32_t *root) {
    return guarded(c, [&]() -> grt_status {
        if (!c) return GRT_ERR_INVALID_ARG;
        if (!c->built) return fail(c, GRT_ERR_NOT_BUILT, "no scene has been built");
        if (c->gpu_tree) return fail(c, GRT_ERR_INVALID_ARG, "a BVH built on the GPU or refitted has no reference tree to export");
        export_tree(c->tree, nodes14, index, root);
        return GRT_OK;
    });
}

struct grt_host_bvh {
    grt::ref_tree tree;
    grt_bvh_stats stats{};
};

}  // extern "C"

const grt::ref_tree &host_tree(const grt_host_bvh *h) { return h->tree; }

extern "C" {

grt_status grt_host_bvh_build(const float *vpos4, uint32_t nv, const uint32_t *tris4, uint32_t nt,
                              const grt_bvh_opts *opts, grt_host_bvh **out) {
    return guarded(nullptr, [&]() -> grt_status {
        if (!out || (nv && !vpos4) || (nt && !tris4)) return GRT_ERR_INVALID_ARG;
        *out = nullptr;
        grt_host_bvh *h = new grt_host_bvh();
        std::string msg;
        auto t0 = std::chrono::steady_clock::now();
        if (!grt::build_reference_bvh(vpos4, nv, tris4, nt, to_build_opts(opts), h->tree, msg)) {
            delete h;
            return GRT_ERR_INVALID_ARG;
        }
        h->stats.build_ms = ms_since(t0);
        h->stats.ref_nodes = (uint32_t)h->tree.nodes.size();
        h->stats.tri_records = (uint32_t)h->tree.index.size();
        h->stats.depth = tree_depth(h->tree);
        *out = h;
        return GRT_OK;
    });
}

grt_status grt_host_bvh_info(const grt_host_bvh *h, grt_bvh_stats *out) {
    if (!h || !out) return GRT_ERR_INVALID_ARG;
    *out = h->stats;
    return GRT_OK;
}

grt_status grt_host_bvh_export(const grt_host_bvh *h, uint32_t *nodes14, uint32_t *index, uint32_t *root) {
    if (!h) return GRT_ERR_INVALID_ARG;
    export_tree(h->tree, nodes14, index, root);
    return GRT_OK;
}

void grt_host_bvh_free(grt_host_bvh *h) { delete h; }

grt_status grt_select_tracer(grt_ctx *c, const char *name) {
    return guarded(c, [&]() -> grt_status {
        if (!c || !name) return GRT_ERR_INVALID_ARG;
        std::string n(name);
        if (n == "default") n = kTracers[0].name;
        // The reference's two other loop shapes, by what they compute per ray: `simple`
        // (rt/cuda/trace-kernels.cu:67-235) is one thread per ray taking one node or leaf per
        // iteration, which is the if-if loop; `dynamic-while-while` (:702-1054) is the while-while
        // loop with lanes refilled when fewer than 20 are active, which is the persistent
        // while-while tracer at its default refill threshold.
        static const char *const aliases[][2] = {{"simple", "if-if"},
                                                 {"simple-alpha", "if-if-alpha"},
                                                 {"dynamic-while-while", "persistent-while-while"},
                                                 {"dynamic-while-while-alpha", "persistent-while-while-alpha"}};
        for (const auto &a : aliases)
            if (n == a[0]) n = a[1];
        for (int i = 0; i < kNumTracers; ++i)
            if (n == kTracers[i].name) {
                c->tracer = i;
                return GRT_OK;
            }
        return fail(c, GRT_ERR_UNKNOWN_TRACER, "there is no tracer named '" + n + "'");
    });
}

grt_status grt_set_tuning(grt_ctx *c, const grt_tuning *t) {
    if (!c || !t) return GRT_ERR_INVALID_ARG;
    if (t->block_threads < 0 || t->block_threads % 32 || t->block_threads > 256 || t->blocks_per_sm < 0 ||
        t->refill_threshold < 0 || t->refill_threshold > 32 || t->refill_period < 0 || t->stack_entries < 0 ||
        t->stack_entries > grt::kStackLarge || t->spec_pend < 0 || t->spec_pend > 3 || t->spec_exit < 0 ||
        t->spec_exit > 32 || t->spec_visits < 0 || t->spec_visits > 16)
        return fail(c, GRT_ERR_INVALID_ARG, "tuning value out of range");
    c->tuning = *t;
    return GRT_OK;
}

grt_status grt_get_tuning(grt_ctx *c, grt_tuning *t) {
    if (!c || !t) return GRT_ERR_INVALID_ARG;
    *t = c->tuning;
    return GRT_OK;
}

timed_call::timed_call(grt_ctx *ctx, int k, cudaStream_t s) : c(ctx), kind(k), st(s) {
    if (!c->timing.enabled) return;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return;
    a = c->timing.take();
    if (a && cudaEventRecord(a, st) != cudaSuccess) {
        c->timing.pool.push_back(a);
        a = nullptr;
    }
}

timed_call::~timed_call() {
    if (!a) return;
    cudaEvent_t b = c->timing.take();
    if (b && cudaEventRecord(b, st) == cudaSuccess) {
        c->timing.pending.push_back({kind, a, b});
        return;
    }
    c->timing.pool.push_back(a);
    if (b) c->timing.pool.push_back(b);
}

grt_status grt_set_timing(grt_ctx *c, int enabled) {
    if (!c) return GRT_ERR_INVALID_ARG;
    c->timing.enabled = enabled != 0;
    return GRT_OK;
}

grt_status grt_timing_stats(grt_ctx *c, grt_timing *out, int reset) {
    return guarded(c, [&]() -> grt_status {
        if (!c) return GRT_ERR_INVALID_ARG;
        device_guard g(c->device);
        timing_state &t = c->timing;
        cudaError_t err = cudaSuccess;
        for (const auto &q : t.pending) {
            float ms = 0.f;
            cudaError_t e = cudaEventSynchronize(q.b);
            if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, q.a, q.b);
            if (e == cudaSuccess) {
                t.calls[q.kind] += 1;
                t.ms[q.kind] += ms;
            } else if (err == cudaSuccess) {
                err = e;
            }
            t.pool.push_back(q.a);
            t.pool.push_back(q.b);
        }
        t.pending.clear();
        if (out)
            for (int k = 0; k < GRT_TIME_KINDS; ++k) {
                out->calls[k] = t.calls[k];
                out->ms[k] = t.ms[k];
            }
        if (reset)
            for (int k = 0; k < GRT_TIME_KINDS; ++k) {
                t.calls[k] = 0;
                t.ms[k] = 0.0;
            }
        return err == cudaSuccess ? GRT_OK : cuda_fail(c, err, "reading the call timers");
    });
}

grt_status grt_trace(grt_ctx *c, const float *rays_dev, grt_hit *hits_dev, uint32_t n, int any_hit,
                     grt_stream_t stream) {
    return guarded(c, [&]() -> grt_status {
        if (!c) return GRT_ERR_INVALID_ARG;
        if (!c->built) return fail(c, GRT_ERR_NOT_BUILT, "grt_trace before a successful grt_build");
        if (n == 0) return GRT_OK;
        if (n > (1u << 31)) return fail(c, GRT_ERR_INVALID_ARG, "more than 2^31 rays in one call");
        if (!rays_dev || !hits_dev || !aligned16(rays_dev) || !aligned16(hits_dev))
            return fail(c, GRT_ERR_INVALID_ARG, "ray and hit buffers must be non-null and 16-byte aligned");
        if (needed_stack(c) > grt::kStackLarge)
            return fail(c, GRT_ERR_BVH_TOO_DEEP, "the selected tracer needs a deeper stack than the kernels have");
        device_guard g(c->device);
        timed_call timer(c, GRT_TIME_TRACE, (cudaStream_t)stream);
        grt::launch_params lp = params_for(c, any_hit != 0);
        cudaError_t e;
        if (kTracers[c->tracer].persistent)
            e = grt::launch_trace_persistent(scene_for(c), (const float4 *)rays_dev, hits_dev, n, any_hit != 0, lp, c->d_err,
                                             c->d_counter, (cudaStream_t)stream);
        else
            e = grt::launch_trace_plain(scene_for(c), (const float4 *)rays_dev, hits_dev, n, any_hit != 0, lp, c->d_err,
                                        (cudaStream_t)stream);
        if (e != cudaSuccess) return cuda_fail(c, e, "launching the traversal kernel");
        return GRT_OK;
    });
}

grt_status grt_set_traversal_counters(grt_ctx *c, unsigned long long *counters_dev) {
    if (!c) return GRT_ERR_INVALID_ARG;
    if (((uintptr_t)counters_dev & 7u) != 0) return fail(c, GRT_ERR_INVALID_ARG, "counters must be 8-byte aligned");
    c->d_trav_counters = counters_dev;
    return GRT_OK;
}

namespace {

// Raises (raise = true) or clears the abort request, on the abort stream. Raising also moves the
// persistent kernels' work counter far past any ray count, so that a running persistent kernel
// finds no more work at its next fetch.
cudaError_t set_abort(grt_ctx *c, bool raise) {
    cudaError_t e = cudaMemcpyAsync(c->d_err + grt::kStatusAbort, c->h_flag + (raise ? 0 : 1), sizeof(unsigned),
                                    cudaMemcpyHostToDevice, c->abort_stream);
    if (e == cudaSuccess && raise)
        e = cudaMemcpyAsync(c->d_err + grt::kStatusCounter, c->h_flag + 2, sizeof(unsigned), cudaMemcpyHostToDevice,
                            c->abort_stream);
    return e == cudaSuccess ? cudaStreamSynchronize(c->abort_stream) : e;
}

// Polls the stream until it is idle or `limit_ms` passes (0: no limit); true when idle.
bool wait_stream(cudaStream_t st, uint32_t limit_ms, cudaError_t &err) {
    const auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        const cudaError_t q = cudaStreamQuery(st);
        if (q == cudaSuccess) return true;
        if (q != cudaErrorNotReady) {
            err = q;
            return false;
        }
        if (limit_ms && ms_since(t0) > limit_ms) return false;
        std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
}

}  // namespace

grt_status grt_abort(grt_ctx *c) {
    if (!c) return GRT_ERR_INVALID_ARG;
    device_guard g(c->device);
    const cudaError_t e = set_abort(c, true);
    return e == cudaSuccess ? GRT_OK : cuda_fail(c, e, "raising the abort request");
}

grt_status grt_check(grt_ctx *c, grt_stream_t stream, uint32_t timeout_ms) {
    return guarded(c, [&]() -> grt_status {
        if (!c) return GRT_ERR_INVALID_ARG;
        device_guard g(c->device);
        cudaStream_t st = (cudaStream_t)stream;
        cudaError_t e = cudaSuccess;
        bool timed_out = false;
        if (!wait_stream(st, timeout_ms, e)) {
            if (e != cudaSuccess) return cuda_fail(c, e, "waiting for the stream");
            // stop the work in flight: persistent kernels finish the rays they hold and take no more
            timed_out = true;
            e = set_abort(c, true);
            if (e != cudaSuccess) return cuda_fail(c, e, "raising the abort request");
            const uint32_t drain_ms = std::max<uint32_t>(2000u, timeout_ms);
            if (!wait_stream(st, drain_ms, e)) {
                if (e != cudaSuccess) return cuda_fail(c, e, "waiting for the aborted stream");
                return fail(c, GRT_ERR_TIMEOUT, "stream did not finish within " + std::to_string(timeout_ms) +
                                                    " ms and had not stopped " + std::to_string(drain_ms) +
                                                    " ms after the abort request, which stays raised");
            }
        }
        unsigned status[grt::kStatusWords] = {0};
        e = cudaMemcpy(status, c->d_err, sizeof(status), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cuda_fail(c, e, "reading the kernel status");
        const unsigned bits = status[grt::kStatusErr];
        const bool raised = status[grt::kStatusAbort] != 0u;
        if (raised) {
            e = set_abort(c, false);  // the stream is idle: later launches run normally again
            if (e != cudaSuccess) return cuda_fail(c, e, "clearing the abort request");
        }
        if (bits) cudaMemset(c->d_err, 0, sizeof(unsigned));
        if (timed_out)
            return fail(c, GRT_ERR_TIMEOUT, "stream did not finish within " + std::to_string(timeout_ms) +
                                                " ms; the work in flight was aborted and its outputs are incomplete");
        if (bits & (grt::ERR_STACK_OVERFLOW | grt::ERR_STEP_LIMIT)) {
            std::string m = "traversal kernel reported:";
            if (bits & grt::ERR_STACK_OVERFLOW) m += " stack overflow";
            if (bits & grt::ERR_STEP_LIMIT) m += " step limit";
            return fail(c, GRT_ERR_TRAVERSAL, m);
        }
        if (raised || (bits & grt::ERR_ABORTED))
            return fail(c, GRT_ERR_ABORTED, "work stopped early after grt_abort; its outputs are incomplete");
        return GRT_OK;
    });
}

grt_status grt_trace_host(grt_ctx *c, const float *rays_host, grt_hit *hits_host, uint32_t n, int any_hit) {
    return guarded(c, [&]() -> grt_status {
        if (!c) return GRT_ERR_INVALID_ARG;
        if (!c->built) return fail(c, GRT_ERR_NOT_BUILT, "grt_trace_host before a successful grt_build");
        if (n == 0) return GRT_OK;
        if (!rays_host || !hits_host) return fail(c, GRT_ERR_INVALID_ARG, "null host buffer");
        device_guard g(c->device);
        const size_t rb = (size_t)n * 32, hb = (size_t)n * 16;
        if (c->stage_bytes < rb + hb) {
            if (c->d_stage) cudaFree(c->d_stage);
            c->d_stage = nullptr;
            c->stage_bytes = 0;
            cudaError_t e = cudaMalloc(&c->d_stage, rb + hb);
            if (e != cudaSuccess) return cuda_fail(c, e, "allocating staging buffers");
            c->stage_bytes = rb + hb;
        }
        float *d_rays = (float *)c->d_stage;
        grt_hit *d_hits = (grt_hit *)((char *)c->d_stage + rb);
        cudaError_t e = cudaMemcpyAsync(d_rays, rays_host, rb, cudaMemcpyHostToDevice, c->stream);
        if (e != cudaSuccess) return cuda_fail(c, e, "copying rays to the device");
        if (any_hit) {  // any-hit leaves beta/gamma as they were, like the reference
            e = cudaMemcpyAsync(d_hits, hits_host, hb, cudaMemcpyHostToDevice, c->stream);
            if (e != cudaSuccess) return cuda_fail(c, e, "copying hits to the device");
        }
        grt_status s = grt_trace(c, d_rays, d_hits, n, any_hit, (grt_stream_t)c->stream);
        if (s != GRT_OK) return s;
        e = cudaMemcpyAsync(hits_host, d_hits, hb, cudaMemcpyDeviceToHost, c->stream);
        if (e != cudaSuccess) return cuda_fail(c, e, "copying hits to the host");
        return grt_check(c, (grt_stream_t)c->stream, 0);
    });
}

}  // extern "C"
