// C-ABI of direct lighting (include/grt.h): the material table with the light distribution
// (the reference's compute_light_distribution, rt/cuda/preprocessing.cpp:17-35) and the
// wavefront and fused forms of the direct-wf steps (direct.cu), light or direction sampling.
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "ctx.hpp"
#include "direct.hpp"

using namespace grt;

namespace {

inline size_t a256(size_t b) { return (b + 255) & ~(size_t)255; }

dl_scene dl_scene_of(const grt_ctx *c) {
    const char *base = (const char *)c->d_dl;
    dl_scene ds;
    ds.vpos = (const float4 *)c->d_vpos;
    ds.tris = (const uint4 *)c->d_tris;
    ds.mats = (const dl::material *)base;
    ds.n_mat = c->dl_n_mat;
    ds.lights = (const uint4 *)(base + c->dl_off_lights);
    ds.lf = (const float *)(base + c->dl_off_f);
    ds.lcdf = (const float *)(base + c->dl_off_cdf);
    ds.n_lights = c->dl_n_lights;
    ds.integral = c->dl_integral;
    return ds;
}

}  // namespace

extern "C" {

grt_status grt_set_material_table(grt_ctx *c, const grt_material *mats, uint32_t n) {
    return guarded(c, [&]() -> grt_status {
        if (!c) return GRT_ERR_INVALID_ARG;
        if (!c->built) return fail(c, GRT_ERR_NOT_BUILT, "grt_set_material_table before a successful build");
        if (n && !mats) return fail(c, GRT_ERR_INVALID_ARG, "null material table");
        device_guard g(c->device);
        // the scene's triangles and vertices, for the lights and their power
        std::vector<float> v((size_t)c->nv * 4);
        std::vector<uint32_t> t((size_t)c->nt * 4);
        cudaError_t e = cudaSuccess;
        if (c->nv) e = cudaMemcpy(v.data(), c->d_vpos, v.size() * 4, cudaMemcpyDeviceToHost);
        if (e == cudaSuccess && c->nt) e = cudaMemcpy(t.data(), c->d_tris, t.size() * 4, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cuda_fail(c, e, "reading the scene back");
        // lights: triangles whose material emits, power = luma(emission * 0.5 |e1 x e2| * pi)
        // (trianglelight::power, libgi/scene.cpp:518-527; luma, libgi/color.h:4-6)
        std::vector<uint32_t> lights;
        std::vector<float> f;
        for (uint32_t i = 0; i < c->nt; ++i) {
            const uint32_t *tri = t.data() + 4 * (size_t)i;
            if (tri[3] >= n) continue;
            const grt_material &m = mats[tri[3]];
            if (m.emissive[0] == 0.f && m.emissive[1] == 0.f && m.emissive[2] == 0.f) continue;
            const float *a = v.data() + 4 * (size_t)tri[0], *b = v.data() + 4 * (size_t)tri[1],
                        *cc = v.data() + 4 * (size_t)tri[2];
            const float e1[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
            const float e2[3] = {cc[0] - a[0], cc[1] - a[1], cc[2] - a[2]};
            const float x[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
            const float len = std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
            float pw[3];
            for (int k = 0; k < 3; ++k) pw[k] = m.emissive[k] * 0.5f * len * dl::kPi;
            f.push_back(0.212671f * pw[0] + 0.715160f * pw[1] + 0.072169f * pw[2]);
            lights.insert(lights.end(), {tri[0], tri[1], tri[2], tri[3]});
        }
        // distribution_1d::build_cdf (libgi/discrete_distributions.cpp:33-45)
        const uint32_t nl = (uint32_t)f.size();
        std::vector<float> cdf(nl + 1, 0.f);
        for (uint32_t i = 1; i <= nl; ++i) cdf[i] = cdf[i - 1] + f[i - 1];
        const float integral = cdf[nl];
        for (uint32_t i = 1; i <= nl; ++i) cdf[i] = integral > 0.f ? cdf[i] / integral : (float)i / (float)nl;
        // one allocation: materials, lights, power, cdf
        const size_t o_l = a256((size_t)std::max(n, 1u) * sizeof(dl::material)), o_f = o_l + a256((size_t)std::max(nl, 1u) * 16),
                     o_c = o_f + a256((size_t)std::max(nl, 1u) * 4), total = o_c + (size_t)(nl + 1) * 4;
        std::vector<char> host(total, 0);
        static_assert(sizeof(dl::material) == sizeof(grt_material), "material layouts differ");
        static_assert(dl::kSampleLight == GRT_DL_SAMPLE_LIGHT && dl::kSampleUniform == GRT_DL_SAMPLE_UNIFORM &&
                          dl::kSampleCosine == GRT_DL_SAMPLE_COSINE,
                      "sampling strategies differ");
        if (n) std::memcpy(host.data(), mats, (size_t)n * sizeof(grt_material));
        if (nl) {
            std::memcpy(host.data() + o_l, lights.data(), (size_t)nl * 16);
            std::memcpy(host.data() + o_f, f.data(), (size_t)nl * 4);
        }
        std::memcpy(host.data() + o_c, cdf.data(), (size_t)(nl + 1) * 4);
        if (c->d_dl) cudaFree(c->d_dl);
        c->d_dl = nullptr;
        e = cudaMalloc(&c->d_dl, total);
        if (e == cudaSuccess) e = cudaMemcpy(c->d_dl, host.data(), total, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            if (c->d_dl) cudaFree(c->d_dl);
            c->d_dl = nullptr;
            return cuda_fail(c, e, "uploading the material table");
        }
        c->dl_n_mat = n;
        c->dl_n_lights = nl;
        c->dl_integral = integral;
        c->dl_off_lights = o_l;
        c->dl_off_f = o_f;
        c->dl_off_cdf = o_c;
        return GRT_OK;
    });
}

grt_status grt_direct(grt_ctx *c, const grt_direct_params *p, const float *rays_dev, uint32_t n, float *fb_dev,
                      grt_stream_t stream) {
    return guarded(c, [&]() -> grt_status {
        if (!c || !p) return GRT_ERR_INVALID_ARG;
        if (!c->built) return fail(c, GRT_ERR_NOT_BUILT, "grt_direct before a successful build");
        if (!c->d_dl) return fail(c, GRT_ERR_INVALID_ARG, "grt_direct needs grt_set_material_table first");
        if (n == 0) return GRT_OK;
        if (!rays_dev || !fb_dev || !aligned16(rays_dev) || !aligned16(fb_dev))
            return fail(c, GRT_ERR_INVALID_ARG, "null or misaligned ray / frame buffer");
        if (p->mode > GRT_DL_FUSED) return fail(c, GRT_ERR_INVALID_ARG, "unknown direct-lighting mode");
        if (p->sampling > GRT_DL_SAMPLE_COSINE || p->reserved != 0)
            return fail(c, GRT_ERR_INVALID_ARG, "unknown direct-lighting sampling strategy");
        if (kTracers[c->tracer].alpha) return fail(c, GRT_ERR_INVALID_ARG, "direct lighting has no alpha-aware form");
        if (needed_stack(c) > kStackLarge) return fail(c, GRT_ERR_BVH_TOO_DEEP, "the BVH needs a deeper stack");
        device_guard g(c->device);
        timed_call timer(c, GRT_TIME_DIRECT, (cudaStream_t)stream);
        const cudaStream_t st = (cudaStream_t)stream;
        const dl_scene ds = dl_scene_of(c);
        const float4 *rays = (const float4 *)rays_dev;
        float4 *fb = (float4 *)fb_dev;
        cudaError_t e = cudaSuccess;
        if (p->mode == GRT_DL_FUSED) {
            const grt_tuning &t = c->tuning;
            const int stack = std::max(needed_stack(c), t.stack_entries);
            e = launch_dl_fused(scene_for(c), ds, rays, n, p->samples, p->seed, p->sampling, 0u, fb,
                                kTracers[c->tracer].order, stack, t.block_threads > 0 ? t.block_threads : 128, c->num_sms,
                                c->d_err, c->d_counter, st);
            return e == cudaSuccess ? GRT_OK : cuda_fail(c, e, "launching the fused direct-lighting kernel");
        }
        // wavefront: hits (16 B), shadow rays (32 B), shadow hits (16 B), light colour + pdf (16 B)
        const size_t need = (size_t)n * 80;
        if (c->dl_scratch_bytes < need) {
            if (c->d_dl_scratch) cudaFree(c->d_dl_scratch);
            c->d_dl_scratch = nullptr;
            c->dl_scratch_bytes = 0;
            e = cudaMalloc(&c->d_dl_scratch, need);
            if (e != cudaSuccess) return cuda_fail(c, e, "allocating the direct-lighting buffers");
            c->dl_scratch_bytes = need;
        }
        char *base = (char *)c->d_dl_scratch;
        grt_hit *hits = (grt_hit *)base;
        float4 *srays = (float4 *)(base + (size_t)n * 16);
        grt_hit *shits = (grt_hit *)(base + (size_t)n * 48);
        float4 *ls = (float4 *)(base + (size_t)n * 64);
        const dev_scene sc = scene_for(c);
        const bool persistent = kTracers[c->tracer].persistent;
        auto trace = [&](const float4 *r, grt_hit *h, bool any) {
            const launch_params lp = params_for(c, any);
            return persistent ? launch_trace_persistent(sc, r, h, n, any, lp, c->d_err, c->d_counter, st)
                              : launch_trace_plain(sc, r, h, n, any, lp, c->d_err, st);
        };
        const bool light = p->sampling == GRT_DL_SAMPLE_LIGHT;  // shadow rays: any hit; directions: closest
        e = trace(rays, hits, false);
        for (uint32_t s = 0; s < p->samples && e == cudaSuccess; ++s) {
            e = launch_dl_sample(ds, rays, hits, n, s, p->seed, p->sampling, srays, ls, fb, st);
            if (e == cudaSuccess) e = trace(srays, shits, light);
            if (e == cudaSuccess) e = launch_dl_integrate(ds, rays, hits, srays, shits, ls, n, p->sampling, fb, st);
        }
        return e == cudaSuccess ? GRT_OK : cuda_fail(c, e, "launching the direct-lighting steps");
    });
}

grt_status grt_hit_albedo(grt_ctx *c, uint32_t mode, const float *rays_dev, uint32_t n, float *fb_dev,
                          grt_stream_t stream) {
    return guarded(c, [&]() -> grt_status {
        if (!c) return GRT_ERR_INVALID_ARG;
        if (!c->built) return fail(c, GRT_ERR_NOT_BUILT, "grt_hit_albedo before a successful build");
        if (!c->d_dl) return fail(c, GRT_ERR_INVALID_ARG, "grt_hit_albedo needs grt_set_material_table first");
        if (n == 0) return GRT_OK;
        if (!rays_dev || !fb_dev || !aligned16(rays_dev) || !aligned16(fb_dev))
            return fail(c, GRT_ERR_INVALID_ARG, "null or misaligned ray / frame buffer");
        if (mode > GRT_DL_FUSED) return fail(c, GRT_ERR_INVALID_ARG, "unknown mode");
        if (kTracers[c->tracer].alpha) return fail(c, GRT_ERR_INVALID_ARG, "albedo shading has no alpha-aware form");
        if (needed_stack(c) > kStackLarge) return fail(c, GRT_ERR_BVH_TOO_DEEP, "the BVH needs a deeper stack");
        device_guard g(c->device);
        timed_call timer(c, GRT_TIME_DIRECT, (cudaStream_t)stream);
        const cudaStream_t st = (cudaStream_t)stream;
        const dl_scene ds = dl_scene_of(c);
        const float4 *rays = (const float4 *)rays_dev;
        float4 *fb = (float4 *)fb_dev;
        cudaError_t e = cudaSuccess;
        if (mode == GRT_DL_FUSED) {
            const grt_tuning &t = c->tuning;
            const int stack = std::max(needed_stack(c), t.stack_entries);
            e = launch_dl_fused(scene_for(c), ds, rays, n, 0u, 0u, GRT_DL_SAMPLE_LIGHT, 1u, fb, kTracers[c->tracer].order,
                                stack, t.block_threads > 0 ? t.block_threads : 128, c->num_sms, c->d_err, c->d_counter,
                                st);
            return e == cudaSuccess ? GRT_OK : cuda_fail(c, e, "launching the fused albedo kernel");
        }
        const size_t need = (size_t)n * 80;  // the direct-lighting scratch; its first n * 16 bytes hold the hits
        if (c->dl_scratch_bytes < need) {
            if (c->d_dl_scratch) cudaFree(c->d_dl_scratch);
            c->d_dl_scratch = nullptr;
            c->dl_scratch_bytes = 0;
            e = cudaMalloc(&c->d_dl_scratch, need);
            if (e != cudaSuccess) return cuda_fail(c, e, "allocating the albedo buffers");
            c->dl_scratch_bytes = need;
        }
        grt_hit *hits = (grt_hit *)c->d_dl_scratch;
        const launch_params lp = params_for(c, false);
        const dev_scene sc = scene_for(c);
        e = kTracers[c->tracer].persistent ? launch_trace_persistent(sc, rays, hits, n, false, lp, c->d_err, c->d_counter, st)
                                           : launch_trace_plain(sc, rays, hits, n, false, lp, c->d_err, st);
        if (e == cudaSuccess) e = launch_add_albedo(ds, hits, n, fb, st);
        return e == cudaSuccess ? GRT_OK : cuda_fail(c, e, "launching the albedo steps");
    });
}

}  // extern "C"
