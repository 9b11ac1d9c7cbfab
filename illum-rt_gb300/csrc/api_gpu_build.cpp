// C-ABI of the GPU builder (include/grt.h): grt_build_device for the context's scene and
// grt_build_scenes_device for a scene set. The kernels are in gpu_build.cu and gpu_build_sah.cu;
// this file owns the allocations, the host threads of a scene-set build and, with the SAH
// method, the grouping of its scenes whose trees are built together, the read-back of each
// tree's depth and stack bound, and the checks the host builder makes (indices in range, depth
// within the traversal stacks, a well-formed tree).
#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <string>
#include <system_error>
#include <thread>
#include <vector>

#include "ctx.hpp"
#include "gpu_build.hpp"
#include "raygen.hpp"
#include "refit.hpp"

using namespace grt;

namespace {

constexpr uint32_t kMaxGpuTris = (1u << 27) - 1;  // leaf references hold 27-bit record indices

// Device buffers of one build call that do not outlive it.
struct build_temps {
    void *scratch = nullptr;
    int32_t *wide_index = nullptr;
    int32_t *info = nullptr;
    void *set = nullptr;  // a scene set's arrays for the SAH trees
    ~build_temps() {
        for (void *p : {scratch, (void *)wide_index, (void *)info, set})
            if (p) cudaFree(p);
    }
};

grt_status check_info(grt_ctx *c, const int32_t *info, const std::string &what) {
    if (info[GB_ERR] & GB_ERR_INDEX) return fail(c, GRT_ERR_INVALID_ARG, what + "a triangle index is beyond the vertex count");
    if (info[GB_ERR] & GB_ERR_TREE) return fail(c, GRT_ERR_TRAVERSAL, what + "the GPU builder made a malformed tree");
    if ((info[GB_ERR] & GB_ERR_DEPTH) || info[GB_DEPTH] > kStackLarge)
        return fail(c, GRT_ERR_BVH_TOO_DEEP,
                    what + "BVH depth " + std::to_string(info[GB_DEPTH]) +
                        " exceeds the largest traversal stack (" + std::to_string(kStackLarge) + ")");
    return GRT_OK;
}

// Host threads (each with a stream) that build the scenes of a scene set concurrently.
constexpr uint32_t kBuildWorkers = 8;

// The streams, scratch and events of those threads; released once their work has finished (and
// on any early return).
struct build_workers {
    std::vector<cudaStream_t> st;
    std::vector<void *> scratch;
    std::vector<cudaEvent_t> done;
    cudaEvent_t ready = nullptr;
    explicit build_workers(int n) : st(n, nullptr), scratch(n, nullptr), done(n, nullptr) {}
    void release() {
        for (size_t w = 0; w < st.size(); ++w) {
            if (st[w]) cudaStreamSynchronize(st[w]);
            if (scratch[w]) cudaFree(scratch[w]);
            if (done[w]) cudaEventDestroy(done[w]);
            if (st[w]) cudaStreamDestroy(st[w]);
            st[w] = nullptr;
            scratch[w] = nullptr;
            done[w] = nullptr;
        }
        if (ready) cudaEventDestroy(ready);
        ready = nullptr;
    }
    ~build_workers() { release(); }
};

// The builder of grt_set_device_builder; the default is the SAH method (trees of the
// reference builder's quality).
int builder_method(int b) {
    switch (b) {
    case GRT_DEVICE_BUILD_LBVH: return GB_METHOD_LBVH;
    case GRT_DEVICE_BUILD_PLOC: return GB_METHOD_PLOC;
    default: return GB_METHOD_SAH;
    }
}

bool bad_mesh(const grt_mesh &m) {
    return (m.nv && !m.vpos4) || (m.nt && !m.tris4) || !aligned16(m.vpos4) || !aligned16(m.tris4) ||
           m.nt > kMaxGpuTris;
}

}  // namespace

extern "C" {

grt_status grt_set_device_builder(grt_ctx *c, int method) {
    if (!c) return GRT_ERR_INVALID_ARG;
    if (method != GRT_DEVICE_BUILD_DEFAULT && method != GRT_DEVICE_BUILD_LBVH && method != GRT_DEVICE_BUILD_PLOC &&
        method != GRT_DEVICE_BUILD_SAH)
        return fail(c, GRT_ERR_INVALID_ARG, "unknown device builder");
    c->device_builder = method;
    return GRT_OK;
}

grt_status grt_set_device_sah_planes(grt_ctx *c, uint32_t planes) {
    if (!c) return GRT_ERR_INVALID_ARG;
    if (planes < 1 || planes > (uint32_t)kMaxSahPlanes)
        return fail(c, GRT_ERR_INVALID_ARG, "SAH planes must be 1..256");
    c->device_planes = (int)planes;
    return GRT_OK;
}

grt_status grt_build_device(grt_ctx *c, const float *vpos4_dev, uint32_t nv, const uint32_t *tris4_dev, uint32_t nt,
                            uint32_t max_tris, grt_stream_t stream) {
    return guarded(c, [&]() -> grt_status {
        if (!c) return GRT_ERR_INVALID_ARG;
        const grt_mesh m{vpos4_dev, nv, tris4_dev, nt};
        if (bad_mesh(m)) return fail(c, GRT_ERR_INVALID_ARG, "null, misaligned or oversized vertex / triangle array");
        if (max_tris < 1 || max_tris > 16) return fail(c, GRT_ERR_INVALID_ARG, "max_tris_per_node must be 1..16");
        device_guard g(c->device);
        timed_call timer(c, GRT_TIME_TREE, (cudaStream_t)stream);
        free_scene(c);
        ++c->scene_generation;
        c->stats = grt_bvh_stats{};
        c->tree = ref_tree();
        const cudaStream_t st = (cudaStream_t)stream;
        const auto t0 = std::chrono::steady_clock::now();

        build_temps tmp;
        const size_t nb = (size_t)std::max(nt, 2u) * 64, rb = (size_t)std::max(nt, 1u) * 48;
        const int method = builder_method(c->device_builder);
        const size_t scratch = gpu_build_scratch_bytes(nt, method);
        cudaError_t e = cudaMalloc(&c->d_nodes, nb);
        if (e == cudaSuccess) e = cudaMalloc(&c->d_recs, rb);
        if (e == cudaSuccess) e = cudaMalloc(&c->d_vpos, std::max<size_t>((size_t)nv * 16, 16));
        if (e == cudaSuccess) e = cudaMalloc(&c->d_tris, std::max<size_t>((size_t)nt * 16, 16));
        if (e == cudaSuccess) e = cudaMalloc(&tmp.scratch, scratch);
        if (e == cudaSuccess) e = cudaMalloc(&tmp.wide_index, (size_t)std::max(nt, 1u) * 4);
        if (e == cudaSuccess) e = cudaMalloc(&tmp.info, 8 * 4);
        if (e == cudaSuccess) e = cudaMalloc(&c->d_parent, (size_t)std::max(nt, 1u) * 4);
        if (e == cudaSuccess && nv) e = cudaMemcpyAsync(c->d_vpos, vpos4_dev, (size_t)nv * 16, cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess && nt) e = cudaMemcpyAsync(c->d_tris, tris4_dev, (size_t)nt * 16, cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess)
            e = gpu_build_binary((const float4 *)c->d_vpos, nv, (const uint4 *)c->d_tris, nt, (int)max_tris, tmp.scratch,
                                 scratch, (float4 *)c->d_nodes, (float4 *)c->d_recs, tmp.wide_index,
                                 (int32_t *)c->d_parent, tmp.info, method, c->device_planes, st);
        int32_t info[8] = {0};
        if (e == cudaSuccess) e = cudaMemcpyAsync(info, tmp.info, sizeof(info), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            free_scene(c);
            return cuda_fail(c, e, "building the BVH on the GPU");
        }
        grt_status s = check_info(c, info, "");
        if (s != GRT_OK) {
            free_scene(c);
            return s;
        }
        const size_t wb = (size_t)std::max(info[GB_WIDE_NODES], 1) * 128;
        e = cudaMalloc(&c->d_nodes4, wb);
        if (e == cudaSuccess) e = gpu_build_wide((const float4 *)c->d_nodes, tmp.wide_index, nt, (float4 *)c->d_nodes4, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            free_scene(c);
            return cuda_fail(c, e, "building the 4-wide BVH on the GPU");
        }
        c->sc.nodes = (const float4 *)c->d_nodes;
        c->sc.records = (const float4 *)c->d_recs;
        c->sc.nodes4 = (const float4 *)c->d_nodes4;
        c->sc.root = nt ? info[GB_ROOT] : 0;
        c->sc.root4 = nt ? info[GB_ROOT4] : 0;
        c->sc.empty = nt == 0 ? 1 : 0;
        c->sc.finite = info[GB_FINITE] ? 1 : 0;
        c->stack_bound4 = (uint32_t)info[GB_BOUND4];
        c->nv = nv;
        c->nt = nt;
        c->depth = (uint32_t)info[GB_DEPTH];
        c->stats.build_ms = ms_since(t0);
        c->stats.inner_nodes = (uint32_t)info[GB_INNER];
        c->stats.tri_records = nt;
        c->stats.depth = c->depth;
        c->stats.device_bytes = nb + rb + wb + (size_t)nv * 16 + (size_t)nt * 16;
        c->d_wide_index = tmp.wide_index;  // kept for refits
        tmp.wide_index = nullptr;
        c->n_links = nt > 1 ? nt - 1 : 0;
        c->n_records = nt;
        c->gpu_tree = true;
        c->built = true;
        return GRT_OK;
    });
}

grt_status grt_refit(grt_ctx *c, const float *vpos4_dev, uint32_t nv, grt_stream_t stream) {
    return guarded(c, [&]() -> grt_status {
        if (!c) return GRT_ERR_INVALID_ARG;
        if (!c->built) return fail(c, GRT_ERR_NOT_BUILT, "grt_refit before a successful build");
        if (nv != c->nv) return fail(c, GRT_ERR_INVALID_ARG, "grt_refit needs the built scene's vertex count");
        if (nv && (!vpos4_dev || !aligned16(vpos4_dev)))
            return fail(c, GRT_ERR_INVALID_ARG, "null or misaligned vertex array");
        if (c->n_links && !c->d_parent) return fail(c, GRT_ERR_INVALID_ARG, "this scene has no refit links");
        device_guard g(c->device);
        timed_call timer(c, GRT_TIME_TREE, (cudaStream_t)stream);
        const cudaStream_t st = (cudaStream_t)stream;
        cudaError_t e = cudaSuccess;
        if (!c->d_refit) e = cudaMalloc(&c->d_refit, 256 + (size_t)std::max(c->n_links, 1u) * 4);
        if (e == cudaSuccess && nv)
            e = cudaMemcpyAsync(c->d_vpos, vpos4_dev, (size_t)nv * 16, cudaMemcpyDeviceToDevice, st);
        refit_args a;
        a.vpos = (const float4 *)c->d_vpos;
        a.tris = (const uint4 *)c->d_tris;
        a.nv = nv;
        a.nt = c->nt;
        a.records = (float4 *)c->d_recs;
        a.n_records = c->sc.empty ? 0 : c->n_records;
        a.nodes = (float4 *)c->d_nodes;
        a.links = (const int32_t *)c->d_parent;
        a.n_nodes = c->sc.empty ? 0 : c->n_links;
        a.root = c->sc.root;
        a.flags = (unsigned *)c->d_refit;
        a.arrive = (unsigned *)((char *)c->d_refit + 256);
        if (e == cudaSuccess) e = launch_refit(a, st);
        // the 4-wide nodes take their children's records from the refitted binary nodes
        if (e == cudaSuccess && a.n_nodes && c->d_wide_index && c->d_nodes4)
            e = gpu_build_wide((const float4 *)c->d_nodes, (const int32_t *)c->d_wide_index, c->n_links + 1,
                               (float4 *)c->d_nodes4, st);
        unsigned flags = 0;
        if (e == cudaSuccess) e = cudaMemcpyAsync(&flags, a.flags, sizeof(flags), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return cuda_fail(c, e, "refitting the BVH");
        ++c->scene_generation;  // captured path-tracing graphs hold the scene's flags
        c->sc.finite = (flags & kRefitNonFinite) ? 0 : 1;
        // the device tree is no longer the reference builder's: nothing to export
        c->tree = ref_tree();
        c->gpu_tree = true;
        if (flags & kRefitBadTree) return fail(c, GRT_ERR_TRAVERSAL, "refit found a malformed tree");
        return GRT_OK;
    });
}

grt_status grt_incoherent_rays(grt_ctx *c, float r1, float r2, uint64_t seed, float *rays_dev, uint32_t n,
                               grt_stream_t stream) {
    if (!c) return GRT_ERR_INVALID_ARG;
    if (!c->built) return fail(c, GRT_ERR_NOT_BUILT, "grt_incoherent_rays before a successful build");
    if (c->nv == 0) return fail(c, GRT_ERR_INVALID_ARG, "the scene has no vertices to place the spheres in");
    if (!(r1 >= 0.f) || !(r2 >= 0.f))  // the reference's check (rt/cuda/base.cpp:125-126)
        return fail(c, GRT_ERR_INVALID_ARG, "incoherence radii must be non-negative");
    if (n == 0) return GRT_OK;
    if (!rays_dev || !aligned16(rays_dev)) return fail(c, GRT_ERR_INVALID_ARG, "null or misaligned ray buffer");
    device_guard g(c->device);
    timed_call timer(c, GRT_TIME_RAYS, (cudaStream_t)stream);
    cudaError_t e = cudaSuccess;
    if (!c->d_extent) e = cudaMalloc(&c->d_extent, 32);
    if (e == cudaSuccess)
        e = launch_incoherent_rays((const float4 *)c->d_vpos, c->nv, r1, r2, seed, (float4 *)rays_dev, n,
                                   (uint32_t *)c->d_extent, (cudaStream_t)stream);
    return e == cudaSuccess ? GRT_OK : cuda_fail(c, e, "generating the incoherent rays");
}

grt_status grt_camera_rays(grt_ctx *c, const grt_camera *cam, uint32_t w, uint32_t h, const float *offsets_dev,
                           int jitter, uint64_t seed, float *rays_dev, grt_stream_t stream) {
    if (!c) return GRT_ERR_INVALID_ARG;
    if (!cam) return fail(c, GRT_ERR_INVALID_ARG, "no camera");
    const uint64_t n = (uint64_t)w * h;
    if (n > 0xFFFFFFFFull) return fail(c, GRT_ERR_INVALID_ARG, "more than 2^32 - 1 rays");
    if (n == 0) return GRT_OK;
    if (!rays_dev || !aligned16(rays_dev)) return fail(c, GRT_ERR_INVALID_ARG, "null or misaligned ray buffer");
    if (offsets_dev && ((uintptr_t)offsets_dev & 7u))
        return fail(c, GRT_ERR_INVALID_ARG, "misaligned offset buffer (needs 8-byte alignment)");
    const float v[11] = {cam->pos[0], cam->pos[1], cam->pos[2], cam->dir[0], cam->dir[1], cam->dir[2],
                         cam->up[0],  cam->up[1],  cam->up[2],  cam->near_w, cam->near_h};
    device_guard g(c->device);
    timed_call timer(c, GRT_TIME_RAYS, (cudaStream_t)stream);
    const cudaError_t e = launch_camera_rays(v, w, h, (const float2 *)offsets_dev, jitter != 0, seed,
                                             (float4 *)rays_dev, (cudaStream_t)stream);
    return e == cudaSuccess ? GRT_OK : cuda_fail(c, e, "generating the camera rays");
}

grt_status grt_build_scenes_device(grt_ctx *c, const grt_mesh *meshes, uint32_t count, uint32_t max_tris,
                                   grt_stream_t stream) {
    return guarded(c, [&]() -> grt_status {
        if (!c) return GRT_ERR_INVALID_ARG;
        if (count == 0 || !meshes) return fail(c, GRT_ERR_INVALID_ARG, "no scenes");
        if (max_tris < 1 || max_tris > 16) return fail(c, GRT_ERR_INVALID_ARG, "max_tris_per_node must be 1..16");
        uint32_t most = 0;
        for (uint32_t i = 0; i < count; ++i) {
            if (bad_mesh(meshes[i]))
                return fail(c, GRT_ERR_INVALID_ARG, "null, misaligned or oversized arrays in scene " + std::to_string(i));
            most = std::max(most, meshes[i].nt);
        }
        device_guard g(c->device);
        timed_call timer(c, GRT_TIME_TREE, (cudaStream_t)stream);
        grt_free_multi(c);
        ++c->scene_generation;
        const cudaStream_t st = (cudaStream_t)stream;
        const auto t0 = std::chrono::steady_clock::now();

        // binary nodes, records and wide indices at 256-byte-aligned offsets of pooled arrays
        auto a256 = [](size_t b) { return (b + 255) & ~(size_t)255; };
        std::vector<std::array<size_t, 3>> off(count);
        size_t tot[3] = {0, 0, 0};
        for (uint32_t i = 0; i < count; ++i) {
            const uint32_t nt = meshes[i].nt;
            const size_t sz[3] = {(size_t)std::max(nt, 2u) * 64, (size_t)std::max(nt, 1u) * 48, (size_t)std::max(nt, 1u) * 4};
            for (int a = 0; a < 3; ++a) {
                off[i][a] = tot[a];
                tot[a] += a256(sz[a]);
            }
        }
        build_temps tmp;
        int32_t *wide_pool = nullptr;
        const int method = builder_method(c->device_builder);
        // With the SAH method the trees of a group of scenes are built together (gpu_build.cu's
        // scene-set phases): groups of consecutive scenes of at most kSahSetMaxTris triangles.
        const bool batched = method == GB_METHOD_SAH;
        std::vector<uint32_t> group_at{0};
        size_t set_bytes = 0;
        if (batched) {
            uint64_t in_group = 0;
            for (uint32_t i = 0; i < count; ++i) {
                if (in_group + meshes[i].nt > kSahSetMaxTris && i > group_at.back()) {
                    set_bytes = std::max(set_bytes, sah_set_carve(nullptr, (uint32_t)in_group, i - group_at.back()).total);
                    group_at.push_back(i);
                    in_group = 0;
                }
                in_group += meshes[i].nt;
            }
            set_bytes = std::max(set_bytes, sah_set_carve(nullptr, (uint32_t)in_group, count - group_at.back()).total);
        }
        group_at.push_back(count);
        const size_t scratch = gpu_build_scratch_bytes(most, batched ? GB_METHOD_LBVH : method);
        cudaError_t e = cudaMalloc(&c->ms.d_nodes, tot[0]);
        if (e == cudaSuccess) e = cudaMalloc(&c->ms.d_recs, tot[1]);
        if (e == cudaSuccess) e = cudaMalloc((void **)&wide_pool, tot[2]);
        // every scene's info, then the error word of the set trees
        if (e == cudaSuccess) e = cudaMalloc(&tmp.info, ((size_t)count + 1) * 8 * 4);
        if (e == cudaSuccess) e = cudaMemsetAsync(tmp.info + 8 * (size_t)count, 0, 8 * 4, st);
        if (e == cudaSuccess && batched) e = cudaMalloc(&tmp.set, set_bytes);
        tmp.wide_index = wide_pool;
        // Per-scene passes run on up to kBuildWorkers host threads, each on a stream of its own with
        // scratch of its own: a build is a chain of short launches (and, for the SAH and PLOC
        // builders, read-backs), so one scene at a time leaves most of the GPU idle.
        const int workers = (int)std::min<uint32_t>(count, kBuildWorkers);
        build_workers W(workers);
        std::vector<cudaStream_t> &wst = W.st;
        std::vector<void *> &wscratch = W.scratch;
        std::vector<cudaEvent_t> &wdone = W.done;
        cudaEvent_t &ready = W.ready;
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ready, cudaEventDisableTiming);
        for (int w = 0; w < workers && e == cudaSuccess; ++w) {
            e = cudaStreamCreateWithFlags(&wst[w], cudaStreamNonBlocking);
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&wdone[w], cudaEventDisableTiming);
            if (e == cudaSuccess) e = cudaMalloc(&wscratch[w], scratch);
        }
        // fn(w, i) for the scenes [i0, i1) on the worker threads; the worker streams start after the
        // work already on `st`, and `st` waits for all of them
        auto on_workers = [&](uint32_t i0, uint32_t i1, auto fn) -> cudaError_t {
            cudaError_t r = cudaEventRecord(ready, st);
            for (int w = 0; w < workers && r == cudaSuccess; ++w) r = cudaStreamWaitEvent(wst[w], ready, 0);
            if (r != cudaSuccess) return r;
            std::atomic<uint32_t> next{i0};
            std::vector<cudaError_t> werr(workers, cudaSuccess);
            auto work = [&](int w) {
                werr[w] = cudaSetDevice(c->device);
                for (uint32_t i; werr[w] == cudaSuccess && (i = next++) < i1;) werr[w] = fn(w, i);
                if (werr[w] == cudaSuccess) werr[w] = cudaEventRecord(wdone[w], wst[w]);
            };
            // the threads that start share the scenes; with none, the calling thread does them
            std::vector<std::thread> pool;
            pool.reserve(workers);
            for (int w = 0; w < workers; ++w) {
                try {
                    pool.emplace_back(work, w);
                } catch (const std::system_error &) {
                    break;
                }
            }
            if (pool.empty()) work(0);
            for (auto &t : pool) t.join();
            const int ran = std::max<int>((int)pool.size(), 1);
            for (int w = 0; w < ran; ++w) {
                if (r == cudaSuccess) r = werr[w];
                if (r == cudaSuccess) r = cudaStreamWaitEvent(st, wdone[w], 0);
            }
            return r;
        };
        auto nodes_of = [&](uint32_t i) { return (float4 *)((char *)c->ms.d_nodes + off[i][0]); };
        auto recs_of = [&](uint32_t i) { return (float4 *)((char *)c->ms.d_recs + off[i][1]); };
        auto wide_of = [&](uint32_t i) { return (int32_t *)((char *)wide_pool + off[i][2]); };
        // one scene on its own (`how`: the builder)
        auto alone = [&](int how) {
            return [&, how](int w, uint32_t i) {
                const grt_mesh &m = meshes[i];
                return gpu_build_binary((const float4 *)m.vpos4, m.nv, (const uint4 *)m.tris4, m.nt, (int)max_tris,
                                        wscratch[w], scratch, nodes_of(i), recs_of(i), wide_of(i), nullptr,
                                        tmp.info + 8 * (size_t)i, how, c->device_planes, wst[w]);
            };
        };
        if (e == cudaSuccess && !batched) e = on_workers(0, count, alone(method));
        for (size_t g = 0; batched && e == cudaSuccess && g + 1 < group_at.size(); ++g) {
            const uint32_t i0 = group_at[g], i1 = group_at[g + 1];
            std::vector<sah_set_scene> table(i1 - i0);
            uint32_t n_g = 0;
            for (uint32_t i = i0; i < i1; ++i) {
                table[i - i0] = sah_set_scene{n_g, meshes[i].nt};
                n_g += meshes[i].nt;
            }
            if (n_g < 2) {  // no scene to split (one triangle at most): the radix-tree path is the same
                e = on_workers(i0, i1, alone(GB_METHOD_LBVH));
                continue;
            }
            const sah_set S = sah_set_carve(tmp.set, n_g, i1 - i0);
            e = on_workers(i0, i1, [&](int w, uint32_t i) {
                const grt_mesh &m = meshes[i];
                return sah_set_prims(S, i - i0, table[i - i0].first, (const float4 *)m.vpos4, m.nv,
                                     (const uint4 *)m.tris4, m.nt, tmp.info + 8 * (size_t)i, wst[w]);
            });
            const uint32_t *order = nullptr;
            if (e == cudaSuccess) e = sah_set_trees(S, table.data(), c->device_planes, &order, tmp.info + 8 * (size_t)count, st);
            if (e == cudaSuccess)
                e = on_workers(i0, i1, [&](int w, uint32_t i) {
                    const grt_mesh &m = meshes[i];
                    return sah_set_finish(S, order, table[i - i0].first, (const float4 *)m.vpos4, m.nv,
                                          (const uint4 *)m.tris4, m.nt, (int)max_tris, wscratch[w], scratch, nodes_of(i),
                                          recs_of(i), wide_of(i), tmp.info + 8 * (size_t)i, wst[w]);
                });
        }
        std::vector<int32_t> info(((size_t)count + 1) * 8, 0);
        if (e == cudaSuccess) e = cudaMemcpyAsync(info.data(), tmp.info, info.size() * 4, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        W.release();  // every worker stream has finished, or the call fails anyway
        if (e != cudaSuccess) {
            grt_free_multi(c);
            return cuda_fail(c, e, "building the scene set on the GPU");
        }
        uint32_t max_depth = 0, max_bound4 = 0;
        std::vector<size_t> off4(count);
        size_t tot4 = 0;
        for (uint32_t i = 0; i < count; ++i) {
            const int32_t *f = info.data() + 8 * (size_t)i;
            grt_status s = check_info(c, f, "scene " + std::to_string(i) + ": ");
            if (s != GRT_OK) {
                grt_free_multi(c);
                return s;
            }
            max_depth = std::max(max_depth, (uint32_t)f[GB_DEPTH]);
            max_bound4 = std::max(max_bound4, (uint32_t)f[GB_BOUND4]);
            off4[i] = tot4;
            tot4 += a256((size_t)std::max(f[GB_WIDE_NODES], 1) * 128);
        }
        if (info[8 * (size_t)count + GB_ERR] & GB_ERR_TREE) {  // the trees built for the whole set
            grt_free_multi(c);
            return fail(c, GRT_ERR_TRAVERSAL, "the GPU builder made a malformed tree");
        }
        e = cudaMalloc(&c->ms.d_nodes4, tot4);
        for (uint32_t i = 0; i < count && e == cudaSuccess; ++i)
            e = gpu_build_wide((const float4 *)((char *)c->ms.d_nodes + off[i][0]),
                               (const int32_t *)((char *)wide_pool + off[i][2]), meshes[i].nt,
                               (float4 *)((char *)c->ms.d_nodes4 + off4[i]), st);
        std::vector<dev_scene> table(count);
        for (uint32_t i = 0; i < count; ++i) {
            const int32_t *f = info.data() + 8 * (size_t)i;
            dev_scene &d = table[i];
            d.nodes = (const float4 *)((char *)c->ms.d_nodes + off[i][0]);
            d.records = (const float4 *)((char *)c->ms.d_recs + off[i][1]);
            d.nodes4 = (const float4 *)((char *)c->ms.d_nodes4 + off4[i]);
            d.root = meshes[i].nt ? f[GB_ROOT] : 0;
            d.root4 = meshes[i].nt ? f[GB_ROOT4] : 0;
            d.empty = meshes[i].nt == 0 ? 1 : 0;
            d.finite = f[GB_FINITE] ? 1 : 0;
        }
        if (e == cudaSuccess) e = cudaMalloc(&c->ms.d_table, count * sizeof(dev_scene));
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(c->ms.d_table, table.data(), count * sizeof(dev_scene), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            grt_free_multi(c);
            return cuda_fail(c, e, "building the 4-wide scene set on the GPU");
        }
        const double build_ms = ms_since(t0);
        c->ms.count = count;
        c->ms.max_depth = max_depth;
        c->ms.max_bound4 = max_bound4;
        c->ms.gpu_tree = true;
        c->ms.stats.resize(count);
        for (uint32_t i = 0; i < count; ++i) {
            const int32_t *f = info.data() + 8 * (size_t)i;
            grt_bvh_stats &s = c->ms.stats[i];
            s = grt_bvh_stats{};
            s.inner_nodes = (uint32_t)f[GB_INNER];
            s.tri_records = meshes[i].nt;
            s.depth = (uint32_t)f[GB_DEPTH];
            s.device_bytes = (size_t)std::max(meshes[i].nt, 2u) * 64 + (size_t)std::max(meshes[i].nt, 1u) * 48 +
                             (size_t)std::max(f[GB_WIDE_NODES], 1) * 128;
            s.build_ms = build_ms;  // wall time of the whole set
        }
        return GRT_OK;
    });
}

}  // extern "C"
