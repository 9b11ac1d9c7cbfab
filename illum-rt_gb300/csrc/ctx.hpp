// The context behind the C-ABI (struct grt_ctx) and helpers shared by the api*.cpp files.
#pragma once
#include <cuda_runtime.h>

#include <array>
#include <atomic>
#include <chrono>
#include <cstring>
#include <exception>
#include <string>
#include <vector>

#include "../../include/grt.h"
#include "bvh_builder.hpp"
#include "grt_internal.hpp"

// Per-call device timing (grt_set_timing): event pairs of the calls since the last read-out,
// and the totals per kind.
struct timing_state {
    bool enabled = false;
    struct pair {
        int kind;
        cudaEvent_t a, b;
    };
    std::vector<pair> pending;
    std::vector<cudaEvent_t> pool;
    uint64_t calls[GRT_TIME_KINDS] = {};
    double ms[GRT_TIME_KINDS] = {};
    cudaEvent_t take() {
        if (!pool.empty()) {
            cudaEvent_t e = pool.back();
            pool.pop_back();
            return e;
        }
        cudaEvent_t e = nullptr;
        return cudaEventCreate(&e) == cudaSuccess ? e : nullptr;
    }
};

struct grt_ctx {
    int device = 0;
    int num_sms = 0;
    std::string err;
    bool built = false;
    bool gpu_tree = false;  // built by grt_build_device or refitted: no reference tree to export
    grt::ref_tree tree;
    grt::dev_scene sc{};
    void *d_nodes = nullptr, *d_recs = nullptr, *d_vpos = nullptr, *d_tris = nullptr, *d_nodes4 = nullptr;
    // refit links: per binary node (parent << 1) | side (-1: root or not in the tree), and the
    // 4-wide node each binary node heads (-1: none); n_links entries each
    void *d_parent = nullptr, *d_wide_index = nullptr;
    void *d_refit = nullptr;  // refit scratch: flags, then one arrival counter per node
    void *d_extent = nullptr;  // six words of scratch for the incoherent-ray generator
    uint32_t n_links = 0, n_records = 0;
    uint32_t nv = 0, nt = 0, depth = 0, stack_bound4 = 0;
    grt_bvh_stats stats{};
    int tracer = 0;  // index into kTracers
    grt_tuning tuning{};
    int device_builder = GRT_DEVICE_BUILD_DEFAULT;  // grt_set_device_builder
    int device_planes = 256;                         // grt_set_device_sah_planes
    timing_state timing;
    unsigned *d_err = nullptr;      // status block (grt_internal.hpp): error bits, counter, abort request
    unsigned *d_counter = nullptr;  // work counter of the persistent kernels (d_err + 1)
    unsigned *h_flag = nullptr;     // pinned {1, 0, kAbortCounter}: the words grt_abort / grt_check write
    cudaStream_t abort_stream = nullptr;  // non-blocking stream of those writes
    void *d_stage = nullptr;        // grt_trace_host staging: rays then hits
    size_t stage_bytes = 0;
    cudaStream_t stream = nullptr;  // grt_trace_host stream
    unsigned long long *d_trav_counters = nullptr;  // grt_set_traversal_counters (caller's memory)
    uint64_t scene_generation = 0;  // bumped by every build (invalidates captured graphs)
    // on-disk cache of reference trees (grt_set_bvh_cache); empty: off
    std::string cache_dir;
    std::atomic<uint64_t> cache_hits{0}, cache_misses{0};
    // texture data of the alpha-aware tracers (grt_set_alpha): one device allocation
    void *d_alpha = nullptr;
    // direct lighting (grt_set_material_table, grt_direct): materials and light distribution in
    // one allocation, per-pixel buffers of the wavefront form in another
    void *d_dl = nullptr;
    uint32_t dl_n_mat = 0, dl_n_lights = 0;
    float dl_integral = 0.f;
    size_t dl_off_lights = 0, dl_off_f = 0, dl_off_cdf = 0;
    void *d_dl_scratch = nullptr;
    size_t dl_scratch_bytes = 0;
    // shading data of the path tracer
    float *d_albedo = nullptr;
    uint32_t n_albedo = 0;
    // scratch arena of the path tracer and the ray-generation steps
    void *d_scratch = nullptr;
    size_t scratch_bytes = 0;
    // captured path-tracing step, replayed while its key matches
    struct graph_cache {
        cudaGraphExec_t exec = nullptr;
        std::vector<uint64_t> key;
    } pt_graph;
    // scene set of the multi-scene path (grt_build_scenes)
    struct multi_set {
        uint32_t count = 0, max_depth = 0, max_bound4 = 0;
        bool gpu_tree = false;  // built by grt_build_scenes_device
        std::vector<grt::ref_tree> trees;
        std::vector<grt_bvh_stats> stats;
        void *d_nodes = nullptr, *d_recs = nullptr, *d_nodes4 = nullptr, *d_vpos = nullptr, *d_tris = nullptr;
        void *d_table = nullptr;    // dev_scene per scene
        void *d_batches = nullptr;  // multi_batch table of the last launch
        uint32_t batch_cap = 0;
    } ms;
};

void grt_free_multi(grt_ctx *c);
const grt::ref_tree &host_tree(const grt_host_bvh *h);

namespace grt {

// The reference build (build_reference_bvh), through the context's on-disk cache when one is
// set (bvh_cache.cpp). Safe to call from several threads at once.
bool build_or_load(grt_ctx *c, const float *vpos4, uint32_t nv, const uint32_t *tris4, uint32_t nt,
                   const build_opts &bo, ref_tree &tree, std::string &err);

struct device_guard {
    int prev = -1;
    explicit device_guard(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) cudaSetDevice(dev);
    }
    ~device_guard() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

// Records an event pair around a call's launches when timing is on (after the context's device
// is current; the stream must not be capturing).
struct timed_call {
    grt_ctx *c;
    int kind;
    cudaStream_t st;
    cudaEvent_t a = nullptr;
    timed_call(grt_ctx *ctx, int k, cudaStream_t s);
    ~timed_call();
};

inline grt_status fail(grt_ctx *c, grt_status s, const std::string &msg) {
    if (c) c->err = msg;
    return s;
}

// The body of a C-ABI entry point, run so that no C++ exception leaves the library: host memory
// or a host thread that could not be had (std::bad_alloc, std::system_error, std::length_error)
// becomes GRT_ERR_OOM, with the reason in grt_last_error where there is a context.
template <class F> grt_status guarded(grt_ctx *c, F &&body) noexcept {
    const char *why = "unknown exception";
    try {
        return body();
    } catch (const std::exception &e) {
        why = e.what();
    } catch (...) {
    }
    if (c) {
        try {
            c->err = std::string("host resources exhausted: ") + why;
        } catch (...) {
            c->err.clear();
        }
    }
    return GRT_ERR_OOM;
}

inline grt_status cuda_fail(grt_ctx *c, cudaError_t e, const char *what) {
    cudaGetLastError();  // clear a non-sticky error so the context stays usable
    return fail(c, e == cudaErrorMemoryAllocation ? GRT_ERR_OOM : GRT_ERR_CUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
}

inline void free_scene(grt_ctx *c) {
    for (void **p : {&c->d_nodes, &c->d_recs, &c->d_vpos, &c->d_tris, &c->d_nodes4, &c->d_alpha, &c->d_dl,
                     &c->d_parent, &c->d_wide_index, &c->d_refit}) {
        if (*p) cudaFree(*p);
        *p = nullptr;
    }
    c->built = false;
    c->gpu_tree = false;
    c->n_links = c->n_records = 0;
}

inline double ms_since(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

// The tracers a context can select (the reference's `raytracer` names for the same loop
// shapes, rt/cuda/platform.cpp:34-56).
// Every loop shape also comes as "<name>-alpha", the alpha-aware variant (the reference
// registers the same pairs, rt/cuda/platform.cpp:34-51).
struct tracer_kind {
    const char *name;
    bool persistent;
    int order;
    bool alpha;
};
inline const tracer_kind kTracers[] = {
    {"while-while", false, WHILE_WHILE, false},
    {"persistent-while-while", true, WHILE_WHILE, false},
    {"if-if", false, IF_IF, false},
    {"persistent-if-if", true, IF_IF, false},
    {"speculative-while-while", false, SPECULATIVE, false},
    {"persistent-speculative-while-while", true, SPECULATIVE, false},
    {"bvh4-speculative-while-while", false, WIDE_SPECULATIVE, false},
    {"persistent-bvh4-speculative-while-while", true, WIDE_SPECULATIVE, false},
    {"while-while-alpha", false, WHILE_WHILE, true},
    {"persistent-while-while-alpha", true, WHILE_WHILE, true},
    {"if-if-alpha", false, IF_IF, true},
    {"persistent-if-if-alpha", true, IF_IF, true},
    {"speculative-while-while-alpha", false, SPECULATIVE, true},
    {"persistent-speculative-while-while-alpha", true, SPECULATIVE, true},
    {"bvh4-speculative-while-while-alpha", false, WIDE_SPECULATIVE, true},
    {"persistent-bvh4-speculative-while-while-alpha", true, WIDE_SPECULATIVE, true}};
inline const int kNumTracers = 16;

// The scene a launch traces: the built scene, with the texture data attached when an
// alpha-aware tracer is selected and grt_set_alpha has supplied it.
inline dev_scene scene_for(const grt_ctx *c) {
    dev_scene s = c->sc;
    s.alpha = kTracers[c->tracer].alpha ? (const alpha_data *)c->d_alpha : nullptr;
    return s;
}

// Stack entries the selected tracer needs on the current scene.
inline int needed_stack(const grt_ctx *c) {
    return kTracers[c->tracer].order == WIDE_SPECULATIVE ? (int)c->stack_bound4 : (int)c->depth;
}

// The speculative parameters of a persistent kernel family: its default with the tuned values
// of grt_tuning in place of the defaults where set.
inline spec_cfg tuned_spec(const grt_tuning &t, spec_cfg d) {
    if (t.spec_pend > 0) d.pend = t.spec_pend;
    if (t.spec_exit > 0) d.exit = t.spec_exit;
    if (t.spec_visits > 0) d.visits = t.spec_visits;
    return d;
}

inline launch_params params_for(grt_ctx *c, bool any_hit) {
    grt::launch_params lp{};
    const grt_tuning &t = c->tuning;
    const int needed = needed_stack(c);
    lp.stack_entries = t.stack_entries > 0 ? t.stack_entries : needed;
    if (lp.stack_entries < needed) lp.stack_entries = needed;
    lp.block_threads = t.block_threads > 0 ? t.block_threads : 128;
    lp.refill_threshold = t.refill_threshold > 0 ? t.refill_threshold : 20;
    lp.refill_period = t.refill_period > 0 ? t.refill_period : 4;
    lp.counters = c->d_trav_counters;
    lp.order = kTracers[c->tracer].order;
    lp.spec = kTracers[c->tracer].persistent ? tuned_spec(t, kSpecPersistent) : kSpecTrace;
    if (kTracers[c->tracer].persistent) {
        int per_sm = t.blocks_per_sm > 0 ? t.blocks_per_sm
                                         : grt::persistent_blocks_per_sm(lp.block_threads, lp.stack_entries, any_hit,
                                                                         lp.order, scene_for(c).alpha != nullptr,
                                                                         lp.spec);
        lp.grid_blocks = per_sm * c->num_sms;
    }
    return lp;
}

inline bool aligned16(const void *p) { return ((uintptr_t)p & 15u) == 0; }

inline build_opts to_build_opts(const grt_bvh_opts *opts) {
    grt_bvh_opts o;
    grt_bvh_opts_default(&o);
    if (opts) o = *opts;
    grt::build_opts bo;
    bo.split = o.split;
    bo.max_tris = o.max_tris_per_node;
    bo.planes = o.number_of_planes;
    bo.esc = o.esc != 0;
    return bo;
}

inline void export_tree(const grt::ref_tree &tree, uint32_t *nodes14, uint32_t *index, uint32_t *root) {
    if (nodes14) {
        for (size_t i = 0; i < tree.nodes.size(); ++i) {
            const grt::ref_node &n = tree.nodes[i];
            uint32_t *o = nodes14 + 14 * i;
            std::memcpy(o + 0, n.lmin, 12);
            std::memcpy(o + 3, n.lmax, 12);
            std::memcpy(o + 6, n.rmin, 12);
            std::memcpy(o + 9, n.rmax, 12);
            std::memcpy(o + 12, &n.link_l, 4);
            std::memcpy(o + 13, &n.link_r, 4);
        }
    }
    if (index) std::memcpy(index, tree.index.data(), tree.index.size() * 4);
    if (root) *root = tree.root;
}

inline uint32_t tree_depth(const grt::ref_tree &tree) {
    // an empty scene is one leaf of count 0, whose link_r = 0 reads as an inner node
    if (tree.index.empty()) return 0;
    uint32_t best = 0;
    std::vector<std::pair<uint32_t, uint32_t>> st = {{tree.root, 0}};
    while (!st.empty()) {
        auto [n, d] = st.back();
        st.pop_back();
        if (d > best) best = d;
        if (tree.nodes[n].inner()) {
            st.push_back({(uint32_t)tree.nodes[n].link_l, d + 1});
            st.push_back({(uint32_t)tree.nodes[n].link_r, d + 1});
        }
    }
    return best;
}

}  // namespace grt
