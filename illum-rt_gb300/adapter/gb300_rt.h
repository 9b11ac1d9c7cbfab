// The drop-in tracer for RTGI's CUDA platform: a wf::cuda::batch_rt (rt/cuda/base.h:403-429)
// whose BVH build and traversal run in libgrt.so through the C-ABI of include/grt.h. A
// maintainer copies this file into the reference tree as rt/cuda/gb300.h and registers the
// tracer in platform::platform (rt/cuda/platform.cpp:34-56) with register_batch_rt.
#pragma once
#include <cstring>  // base.h calls memset without including it

#include "base.h"
#include "grt.h"  // include/grt.h of this repository

#include <stdexcept>

namespace wf::cuda {

// A wf::cuda::batch_rt (rt/cuda/base.h:403-429) whose build and traversal run in libgrt.
struct gb300_rt : public batch_rt {
    grt_ctx *ctx = nullptr;

    explicit gb300_rt(const char *tracer) {
        if (grt_create(nullptr, &ctx) != GRT_OK) throw std::runtime_error("grt_create failed");
        if (grt_select_tracer(ctx, tracer) != GRT_OK) throw std::logic_error(grt_last_error(ctx));
    }
    ~gb300_rt() { grt_destroy(ctx); }

    // same inputs as batch_rt::build (rt/cuda/base.cpp:88-117): host copies of the scene
    void build(scenedata *scene) override {
        scene->triangles.download();
        scene->vertex_pos.download();
        grt_bvh_opts o;
        grt_bvh_opts_default(&o);  // SAH, 16 planes, ESC: the CUDA platform's settings
        o.max_tris_per_node = bvh_max_tris_per_node;
        o.split = bvh_type == "om" ? GRT_SPLIT_OM : bvh_type == "sm" ? GRT_SPLIT_SM : GRT_SPLIT_SAH;
        grt_status s = grt_build(ctx, reinterpret_cast<const float *>(scene->vertex_pos.host_data.data()),
                                 scene->vertex_pos.host_data.size(),
                                 reinterpret_cast<const uint32_t *>(scene->triangles.host_data.data()),
                                 scene->triangles.host_data.size(), &o);
        scene->triangles.free_host_data();
        if (s != GRT_OK) throw std::runtime_error(grt_last_error(ctx));
    }

    // batch_rt::compute_hit (rt/cuda/base.h:422-428): rays float4[2n] in, tri_is[n] out
    void compute_hit(bool anyhit) override {
        const uint32_t n = rd->w * rd->h;
        grt_status s = grt_trace(ctx, reinterpret_cast<const float *>(rd->rays.device_memory),
                                 reinterpret_cast<grt_hit *>(rd->intersections.device_memory), n, anyhit, nullptr);
        if (s == GRT_OK) s = grt_check(ctx, nullptr, 0);  // synchronous like the reference tracers
        if (s != GRT_OK) throw std::runtime_error(grt_last_error(ctx));
    }
};

}  // namespace wf::cuda
