// C-ABI of the multi-scene path (include/grt.h): many independent scenes built in parallel on
// the host, uploaded into pooled device arrays, and traced with uneven ray batches in one
// persistent launch.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <thread>

#include "ctx.hpp"
#include "multi.hpp"

using namespace grt;

void grt_free_multi(grt_ctx *c) {
    for (void **p : {&c->ms.d_nodes, &c->ms.d_recs, &c->ms.d_nodes4, &c->ms.d_vpos, &c->ms.d_tris, &c->ms.d_table,
                     &c->ms.d_batches}) {
        if (*p) cudaFree(*p);
        *p = nullptr;
    }
    c->ms = grt_ctx::multi_set();
}

extern "C" {

grt_status grt_build_scenes(grt_ctx *c, const grt_mesh *meshes, uint32_t count, const grt_bvh_opts *opts) {
    return guarded(c, [&]() -> grt_status {
        if (!c) return GRT_ERR_INVALID_ARG;
        if (count == 0 || !meshes) return fail(c, GRT_ERR_INVALID_ARG, "no scenes");
        for (uint32_t i = 0; i < count; ++i)
            if ((meshes[i].nv && !meshes[i].vpos4) || (meshes[i].nt && !meshes[i].tris4))
                return fail(c, GRT_ERR_INVALID_ARG, "null vertex or triangle array in scene " + std::to_string(i));
        device_guard g(c->device);
        grt_free_multi(c);
        ++c->scene_generation;
        build_opts bo = to_build_opts(opts);
        bo.threads = 1;  // scenes are built concurrently, one thread each

        auto t0 = std::chrono::steady_clock::now();
        std::vector<ref_tree> trees(count);
        std::vector<flat_bvh> flats(count);
        std::vector<flat_bvh4> wides(count);
        std::vector<std::string> errs(count);
        std::vector<uint8_t> ok(count, 0);
        std::vector<uint32_t> order(count);
        for (uint32_t i = 0; i < count; ++i) order[i] = i;
        std::sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return meshes[a].nt > meshes[b].nt; });
        std::atomic<uint32_t> next{0};
        auto worker = [&]() {
            for (uint32_t k; (k = next++) < count;) {
                const uint32_t i = order[k];
                const grt_mesh &m = meshes[i];
                ok[i] = build_or_load(c, m.vpos4, m.nv, m.tris4, m.nt, bo, trees[i], errs[i]) &&
                        flatten_bvh(trees[i], m.vpos4, m.tris4, flats[i], errs[i]) &&
                        flatten_bvh4(trees[i], flats[i], wides[i], errs[i]);
            }
        };
        const uint32_t nthreads = std::max(1u, std::min(count, std::thread::hardware_concurrency()));
        std::vector<std::thread> pool;
        for (uint32_t t = 0; t < nthreads; ++t) pool.emplace_back(worker);
        for (auto &t : pool) t.join();
        for (uint32_t i = 0; i < count; ++i)
            if (!ok[i]) return fail(c, GRT_ERR_INVALID_ARG, "scene " + std::to_string(i) + ": " + errs[i]);
        const double build_ms = ms_since(t0);

        // pooled layout
        t0 = std::chrono::steady_clock::now();
        size_t tot[5] = {0, 0, 0, 0, 0};  // nodes, records, nodes4, vpos, tris (bytes)
        std::vector<std::array<size_t, 5>> off(count);
        uint32_t max_depth = 0, max_bound4 = 0;
        for (uint32_t i = 0; i < count; ++i) {
            const size_t sz[5] = {flats[i].nodes.size() * 4, flats[i].records.size() * 4, wides[i].nodes.size() * 4,
                                  (size_t)meshes[i].nv * 16, (size_t)meshes[i].nt * 16};
            for (int a = 0; a < 5; ++a) {
                off[i][a] = tot[a];
                tot[a] += (sz[a] + 255) & ~(size_t)255;
            }
            max_depth = std::max(max_depth, flats[i].depth);
            max_bound4 = std::max(max_bound4, wides[i].stack_bound);
        }
        cudaError_t e = cudaSuccess;
        void **pools[5] = {&c->ms.d_nodes, &c->ms.d_recs, &c->ms.d_nodes4, &c->ms.d_vpos, &c->ms.d_tris};
        for (int a = 0; a < 5 && e == cudaSuccess; ++a) e = cudaMalloc(pools[a], std::max<size_t>(tot[a], 256));
        std::vector<dev_scene> table(count);
        for (uint32_t i = 0; i < count && e == cudaSuccess; ++i) {
            const void *src[5] = {flats[i].nodes.data(), flats[i].records.data(), wides[i].nodes.data(), meshes[i].vpos4,
                                  meshes[i].tris4};
            const size_t sz[5] = {flats[i].nodes.size() * 4, flats[i].records.size() * 4, wides[i].nodes.size() * 4,
                                  (size_t)meshes[i].nv * 16, (size_t)meshes[i].nt * 16};
            for (int a = 0; a < 5 && e == cudaSuccess; ++a)
                if (sz[a]) e = cudaMemcpy((char *)*pools[a] + off[i][a], src[a], sz[a], cudaMemcpyHostToDevice);
            bool finite = true;
            for (size_t q = 0; q < (size_t)meshes[i].nv && finite; ++q)
                for (int k = 0; k < 3; ++k) finite = finite && std::isfinite(meshes[i].vpos4[4 * q + k]);
            dev_scene &d = table[i];
            d.nodes = (const float4 *)((char *)c->ms.d_nodes + off[i][0]);
            d.records = (const float4 *)((char *)c->ms.d_recs + off[i][1]);
            d.nodes4 = (const float4 *)((char *)c->ms.d_nodes4 + off[i][2]);
            d.root = flats[i].root;
            d.root4 = wides[i].root;
            d.empty = flats[i].empty ? 1 : 0;
            d.finite = finite ? 1 : 0;
        }
        if (e == cudaSuccess) e = cudaMalloc(&c->ms.d_table, count * sizeof(dev_scene));
        if (e == cudaSuccess) e = cudaMemcpy(c->ms.d_table, table.data(), count * sizeof(dev_scene), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            grt_free_multi(c);
            return cuda_fail(c, e, "uploading the scenes");
        }
        const double upload_ms = ms_since(t0);
        c->ms.count = count;
        c->ms.max_depth = max_depth;
        c->ms.max_bound4 = max_bound4;
        c->ms.stats.resize(count);
        for (uint32_t i = 0; i < count; ++i) {
            grt_bvh_stats &s = c->ms.stats[i];
            s = grt_bvh_stats{};
            s.ref_nodes = (uint32_t)trees[i].nodes.size();
            s.inner_nodes = flats[i].inner;
            s.tri_records = (uint32_t)trees[i].index.size();
            s.depth = flats[i].depth;
            s.device_bytes = flats[i].nodes.size() * 4 + flats[i].records.size() * 4 + wides[i].nodes.size() * 4 +
                             (size_t)meshes[i].nv * 16 + (size_t)meshes[i].nt * 16;
            s.build_ms = build_ms;  // wall time of the whole parallel build
            s.upload_ms = upload_ms;
        }
        c->ms.trees = std::move(trees);
        return GRT_OK;
    });
}

grt_status grt_scene_info(grt_ctx *c, uint32_t scene, grt_bvh_stats *out) {
    if (!c || !out) return GRT_ERR_INVALID_ARG;
    if (scene >= c->ms.count) return fail(c, GRT_ERR_INVALID_ARG, "no such scene");
    *out = c->ms.stats[scene];
    return GRT_OK;
}

grt_status grt_export_scene_bvh(grt_ctx *c, uint32_t scene, uint32_t *nodes14, uint32_t *index, uint32_t *root) {
    return guarded(c, [&]() -> grt_status {
        if (!c) return GRT_ERR_INVALID_ARG;
        if (scene >= c->ms.count) return fail(c, GRT_ERR_INVALID_ARG, "no such scene");
        if (c->ms.gpu_tree) return fail(c, GRT_ERR_INVALID_ARG, "a scene set built on the GPU has no reference trees to export");
        export_tree(c->ms.trees[scene], nodes14, index, root);
        return GRT_OK;
    });
}

grt_status grt_trace_multi(grt_ctx *c, const grt_ray_batch *batches, uint32_t count, int any_hit,
                           grt_stream_t stream) {
    return guarded(c, [&]() -> grt_status {
        if (!c) return GRT_ERR_INVALID_ARG;
        if (c->ms.count == 0) return fail(c, GRT_ERR_NOT_BUILT, "grt_trace_multi before grt_build_scenes");
        if (count == 0) return GRT_OK;
        if (!batches) return fail(c, GRT_ERR_INVALID_ARG, "null batch table");
        std::vector<multi_batch> tab(count);
        uint64_t total = 0;
        for (uint32_t b = 0; b < count; ++b) {
            const grt_ray_batch &x = batches[b];
            if (x.scene >= c->ms.count) return fail(c, GRT_ERR_INVALID_ARG, "batch " + std::to_string(b) + ": no such scene");
            if (x.n && (!x.rays_dev || !x.hits_dev || !aligned16(x.rays_dev) || !aligned16(x.hits_dev)))
                return fail(c, GRT_ERR_INVALID_ARG, "batch " + std::to_string(b) + ": null or misaligned buffer");
            tab[b] = {(const float4 *)x.rays_dev, x.hits_dev, (uint32_t)total, x.scene, x.n, 0};
            total += x.n;
        }
        if (total > (1ull << 31)) return fail(c, GRT_ERR_INVALID_ARG, "more than 2^31 rays in one call");
        if (kTracers[c->tracer].alpha)
            return fail(c, GRT_ERR_INVALID_ARG, "alpha-aware tracing of scene sets is not supported");
        const int order = kTracers[c->tracer].order;
        const int needed = order == WIDE_SPECULATIVE ? (int)c->ms.max_bound4 : (int)c->ms.max_depth;
        if (needed > kStackLarge)
            return fail(c, GRT_ERR_BVH_TOO_DEEP, "a scene needs a deeper stack than the kernels have");
        device_guard g(c->device);
        timed_call timer(c, GRT_TIME_TRACE_MULTI, (cudaStream_t)stream);
        if (c->ms.batch_cap < count) {
            if (c->ms.d_batches) cudaFree(c->ms.d_batches);
            c->ms.d_batches = nullptr;
            c->ms.batch_cap = 0;
            cudaError_t e = cudaMalloc(&c->ms.d_batches, count * sizeof(multi_batch));
            if (e != cudaSuccess) return cuda_fail(c, e, "allocating the batch table");
            c->ms.batch_cap = count;
        }
        // pageable source: the copy is staged before the call returns, so `tab` may go out of scope
        cudaError_t e = cudaMemcpyAsync(c->ms.d_batches, tab.data(), count * sizeof(multi_batch), cudaMemcpyHostToDevice,
                                        (cudaStream_t)stream);
        if (e != cudaSuccess) return cuda_fail(c, e, "copying the batch table");
        launch_params lp{};
        const grt_tuning &t = c->tuning;
        lp.order = order;
        lp.spec = tuned_spec(t, kSpecPersistent);
        lp.stack_entries = std::max(t.stack_entries, needed);
        lp.block_threads = t.block_threads > 0 ? t.block_threads : 128;
        lp.refill_threshold = t.refill_threshold > 0 ? t.refill_threshold : 20;
        lp.refill_period = t.refill_period > 0 ? t.refill_period : 4;
        lp.grid_blocks =
            (t.blocks_per_sm > 0 ? t.blocks_per_sm : multi_blocks_per_sm(lp.block_threads, lp.stack_entries, order, lp.spec)) *
            c->num_sms;
        e = launch_trace_multi((const dev_scene *)c->ms.d_table, (const multi_batch *)c->ms.d_batches, count,
                               (uint32_t)total, any_hit != 0, lp, c->d_err, c->d_counter, (cudaStream_t)stream);
        return e == cudaSuccess ? GRT_OK : cuda_fail(c, e, "launching the multi-scene kernel");
    });
}

}  // extern "C"
