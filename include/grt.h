/*
 * grt.h — C-ABI of the GB300 batch ray-traversal library (libgrt.so).
 *
 * The library replaces the CUDA batch tracers of RTGI (lwolf98/illum-rt). In the reference a
 * wavefront algorithm calls a pluggable `wf::batch_ray_tracer` (libgi/wavefront-rt.h:145-149)
 * whose CUDA specialisation `wf::cuda::batch_rt` (rt/cuda/base.h:403-429) builds a BVH on the
 * host (rt/cuda/base.cpp:88-117) and launches traversal kernels over device ray buffers
 * (rt/cuda/tracers.cu:57-294). This header exposes the same operations over plain pointers and
 * sizes so that a thin adapter class deriving from wf::cuda::batch_rt can drop in for that path.
 *
 * Data layouts are the reference's device layouts:
 *   vertex positions : float4 per vertex (x, y, z, 1)              rt/cuda/base.cpp:57-66
 *   triangles        : uint4 per triangle (a, b, c, material id)   rt/cuda/base.cpp:49-53
 *   rays             : two float4 per ray, (o.xyz, t_min), (d.xyz, t_max)
 *                                                                  rt/cuda/base.h:337, kernels.cu:52-60
 *   hits             : grt_hit per ray, identical to wf::cuda::tri_is (rt/cuda/base.h:32-41)
 *
 * Results: closest hits are those of the reference CPU tracer binary_bvh_tracer::closest_hit
 * (rt/cpu/bvh2.cpp:71-137) on the same BVH: same triangle, bit-identical t, beta, gamma (the
 * ray/triangle test is the reference's Cramer test, libgi/intersect.h:19-74, evaluated with
 * the same IEEE operations). A miss is t = FLT_MAX, ref = 0. Any-hit results use the CPU
 * platform's encoding (rt/cpu/wavefront.cpp:60-70): occluded rays get ref = 0xFFFFFFFF and
 * t = 4294967296.0f; the others t = FLT_MAX, ref = 0; beta and gamma are not written.
 *
 * Errors are status codes, never exceptions (host memory or a host thread that cannot be had
 * is GRT_ERR_OOM), and the library never resets the device (the reference's check_cuda_error
 * calls cudaDeviceReset, rt/cuda/cuda-helpers.cpp:5-12).
 * All launches are stream-ordered and asynchronous; grt_check() synchronises the stream and
 * reports errors that kernels flagged (stack overflow, step limit). A context is not
 * thread-safe; use one context per host thread.
 */
#ifndef GRT_H
#define GRT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GRT_VERSION_MAJOR 1
#define GRT_VERSION_MINOR 2

/* A cudaStream_t. NULL means the legacy default stream. */
typedef struct CUstream_st *grt_stream_t;
typedef struct grt_ctx grt_ctx;

typedef enum grt_status {
    GRT_OK = 0,
    GRT_ERR_INVALID_ARG = 1,    /* bad pointer, size or option */
    GRT_ERR_OOM = 2,            /* device or pinned host allocation failed */
    GRT_ERR_CUDA = 3,           /* a CUDA runtime call failed (message in grt_last_error) */
    GRT_ERR_TIMEOUT = 4,        /* grt_check gave up waiting for the stream */
    GRT_ERR_BVH_TOO_DEEP = 5,   /* the BVH needs a deeper stack than any kernel variant has */
    GRT_ERR_NOT_BUILT = 6,      /* trace called before a successful build */
    GRT_ERR_TRAVERSAL = 7,      /* a kernel flagged a stack overflow or hit its step limit */
    GRT_ERR_UNKNOWN_TRACER = 8, /* grt_select_tracer: no tracer of that name */
    GRT_ERR_NO_DEVICE = 9,      /* no CUDA device of the requested ordinal */
    GRT_ERR_TOO_LARGE = 10,     /* input exceeds the fixed capacity of grt_compact_hits_static */
    GRT_ERR_ABORTED = 11        /* work stopped early after grt_abort; its outputs are incomplete */
} grt_status;

/* One hit record, 16 bytes, the layout of wf::cuda::tri_is (rt/cuda/base.h:32-41).
 * `ref` is the index of the triangle in the triangle array given to grt_build. */
typedef struct grt_hit {
    float t, beta, gamma;
    uint32_t ref;
} grt_hit;

typedef struct grt_config {
    int device;         /* CUDA device ordinal */
    uint32_t reserved;  /* must be 0 */
} grt_config;

/* BVH builder options: the `bvh type` / `bvh max_tris` commands of the CUDA tracer
 * (rt/cuda/base.cpp:134-153). Defaults (grt_bvh_opts_default) are the reference's CUDA
 * build: SAH with 16 planes, at most 4 triangles per leaf, early split clipping on. */
enum { GRT_SPLIT_OM = 0, GRT_SPLIT_SM = 1, GRT_SPLIT_SAH = 2 };
typedef struct grt_bvh_opts {
    int split;             /* GRT_SPLIT_SAH, GRT_SPLIT_SM or GRT_SPLIT_OM */
    int max_tris_per_node; /* 1..16 */
    int number_of_planes;  /* SAH candidate planes, >= 1 */
    int esc;               /* early split clipping, 0 or 1 */
} grt_bvh_opts;

typedef struct grt_bvh_stats {
    uint32_t ref_nodes;     /* nodes of the reference layout (inner + leaf) */
    uint32_t inner_nodes;   /* 64-byte device nodes */
    uint32_t tri_records;   /* 48-byte device triangle records (ESC duplicates included) */
    uint32_t depth;         /* edges from the root to the deepest leaf */
    uint64_t device_bytes;  /* nodes + records + triangles + vertices held on the device */
    double build_ms;        /* host SAH/ESC build */
    double flatten_ms;      /* host flattening */
    double upload_ms;       /* host-to-device copies */
} grt_bvh_stats;

/* Launch parameters picked by the autotuner (or by hand). Zero fields mean "default". The
 * reference's counterparts are compile-time constants of its CUDA tracers (BATCH_SIZE,
 * DYNAMIC_FETCH_THRESHOLD, STACK_SIZE; rt/cuda/trace-kernels.cu:6-8). */
typedef struct grt_tuning {
    int block_threads;     /* threads per block (multiple of 32) */
    int blocks_per_sm;     /* persistent kernels: resident blocks per SM */
    int refill_threshold;  /* persistent kernels: refill a warp when fewer lanes are active */
    int refill_period;     /* persistent kernels: traversal steps between refill checks */
    int stack_entries;     /* traversal stack entries per thread (shared memory); 0 = the BVH's
                              depth, larger values up to 64 allowed, smaller ones raised to it */
    /* Speculative loop order of the persistent kernels (fused path tracer, persistent traces,
     * scene sets); 0 = the measured default of each kernel family: */
    int spec_pend;         /* leaves a lane may postpone before the warp's leaf phase, 1..3 */
    int spec_exit;         /* the warp leaves its node phase once at most this many lanes still
                              search for their first leaf, 1..32 */
    int spec_visits;       /* node visits per lane between two warp votes, 1..16 */
} grt_tuning;

/* ---- context ------------------------------------------------------------------------ */

/* Version as major*1000 + minor. */
int grt_version(void);

/* Creates a context on config->device (NULL = device 0). */
grt_status grt_create(const grt_config *config, grt_ctx **out);
grt_status grt_destroy(grt_ctx *ctx);

/* Message of the last error on this context ("" if none). Valid until the next call. */
const char *grt_last_error(const grt_ctx *ctx);

/* Fills opts with the reference CUDA defaults (SAH, 16 planes, 4 per leaf, ESC on). */
void grt_bvh_opts_default(grt_bvh_opts *opts);

/* ---- build (wf::cuda::batch_rt::build, rt/cuda/base.cpp:88-117) --------------------- */

/* Builds the BVH of one scene from HOST arrays with the reference's CPU SAH/SM/OM builder
 * and early split clipping (rt/cpu/bvh-ctor.h:96-503), flattens it into the device layout and
 * uploads it. Replaces any previous scene of the context. opts may be NULL (defaults). */
grt_status grt_build(grt_ctx *ctx, const float *vpos4, uint32_t nv, const uint32_t *tris4, uint32_t nt,
                     const grt_bvh_opts *opts);

grt_status grt_bvh_info(grt_ctx *ctx, grt_bvh_stats *out);

/* Copies the BVH of the current scene in the reference's layout: `nodes14` receives
 * stats.ref_nodes records of 14 words (box_l.min xyz, box_l.max xyz, box_r.min xyz,
 * box_r.max xyz as float bits, link_l, link_r; bbvh_node, rt/cpu/bvh.h:42-52) and `index`
 * receives stats.tri_records triangle ids (::bvh::index, rt/cpu/bvh.h:58-63). Either may be
 * NULL. Used to check the builder against the reference. */
grt_status grt_export_bvh(grt_ctx *ctx, uint32_t *nodes14, uint32_t *index, uint32_t *root);

/* Host-only access to the builder (no device needed): builds the reference BVH and keeps it
 * in host memory so that its nodes can be compared with the reference's. */
typedef struct grt_host_bvh grt_host_bvh;
grt_status grt_host_bvh_build(const float *vpos4, uint32_t nv, const uint32_t *tris4, uint32_t nt,
                              const grt_bvh_opts *opts, grt_host_bvh **out);
/* ref_nodes, tri_records and depth of the host BVH; build_ms of its construction. */
grt_status grt_host_bvh_info(const grt_host_bvh *bvh, grt_bvh_stats *out);

/* On-disk cache of built trees. No counterpart in the reference, which builds every scene
 * again on each start (its tracer can only export boxes, rt/cpu/bvh2.cpp:228-285). With a
 * directory set, grt_build and grt_build_scenes first look for a file named by a 128-bit hash
 * of the vertex and triangle arrays and the builder options; a file that is missing, from
 * other inputs or damaged costs one build, after which the tree is written there (under a
 * temporary name, then renamed). The cached tree is the reference builder's, so results are
 * unchanged. NULL or "" switches the cache off. */
grt_status grt_set_bvh_cache(grt_ctx *ctx, const char *directory);
/* Builds served from the cache (hits) and built and stored (misses) since the context was made. */
grt_status grt_bvh_cache_stats(const grt_ctx *ctx, uint64_t *hits, uint64_t *misses);

/* The reference tracer's `bvh export <depth> <file.obj>` (rt/cpu/bvh2.cpp:228-283): the child
 * boxes of the inner nodes above `max_depth` as OBJ quads, grouped by level, in the reference's
 * order and number format. */
grt_status grt_export_bvh_obj(grt_ctx *ctx, int max_depth, const char *path);

/* The reference tracer's `bvh statistics` (rt/cpu/bvh2.cpp:286-317), computed the same way
 * (the maximum is only updated by a leaf that is not a new minimum; the median of an even
 * number of leaves averages positions n/2 and n/2 + 1, so two leaves are an error). */
typedef struct grt_leaf_stats {
    uint32_t leaves;
    int32_t min_tris, max_tris;
    uint32_t avg_tris;   /* integer division, as printed by the reference */
    int32_t median_tris;
} grt_leaf_stats;
grt_status grt_bvh_leaf_stats(grt_ctx *ctx, grt_leaf_stats *out);
/* The same two for a host-only BVH (no device needed). */
grt_status grt_host_bvh_export_obj(const grt_host_bvh *bvh, int max_depth, const char *path);
grt_status grt_host_bvh_leaf_stats(const grt_host_bvh *bvh, grt_leaf_stats *out);
grt_status grt_host_bvh_export(const grt_host_bvh *bvh, uint32_t *nodes14, uint32_t *index, uint32_t *root);
void grt_host_bvh_free(grt_host_bvh *bvh);

/* ---- tracer selection (platform::select / `raytracer <name>`, rt/cuda/platform.cpp:102-131) */

/* Names: "while-while" (default), "if-if" and "speculative-while-while": one thread per ray,
 * in the loop orders of the reference's tracers of those names; "bvh4-speculative-while-while":
 * the speculative order over the BVH collapsed into 4-wide nodes; the same names prefixed with
 * "persistent-": persistent warps with dynamic ray fetch. The loop order of the selected tracer
 * is also the one grt_pathtrace uses. The if-if and while-while orders give results identical
 * to the reference CPU tracer; the speculative orders may differ from it in near-ties only (a
 * different triangle whose t is within a few ulps of the reference's). Every name also comes
 * with the suffix "-alpha" (alpha-aware, grt_set_alpha). The reference's "simple" and
 * "dynamic-while-while" (and their "-alpha" forms) are accepted too and select "if-if" and
 * "persistent-while-while", the loops that compute what they compute. Unknown name:
 * GRT_ERR_UNKNOWN_TRACER. */
grt_status grt_select_tracer(grt_ctx *ctx, const char *name);
grt_status grt_set_tuning(grt_ctx *ctx, const grt_tuning *tuning);
grt_status grt_get_tuning(grt_ctx *ctx, grt_tuning *tuning);

/* ---- trace (batch_rt::compute_closest_hit / compute_any_hit, rt/cuda/base.h:422-428) ---- */

/* Traces n rays from DEVICE buffers: rays_dev holds 2n float4, hits_dev n grt_hit (16-byte
 * aligned). Asynchronous on `stream`; call grt_check to wait and collect kernel errors. */
grt_status grt_trace(grt_ctx *ctx, const float *rays_dev, grt_hit *hits_dev, uint32_t n, int any_hit,
                     grt_stream_t stream);

/* Same as grt_trace from HOST buffers: copies the rays in, traces, copies the hits out and
 * waits. Uses context-owned device and pinned staging buffers. */
grt_status grt_trace_host(grt_ctx *ctx, const float *rays_host, grt_hit *hits_host, uint32_t n, int any_hit);

/* Traversal statistics: while counters_dev (three uint64 in device memory) is set, every ray
 * traced by the one-thread-per-ray kernel (tracer "while-while", and the per-bounce traces of
 * GRT_PT_WAVEFRONT) adds 1 to counters_dev[0], its inner-node visits to [1] and its triangle
 * tests to [2]. The counting kernel is a separate, slower variant; NULL switches it off. */
grt_status grt_set_traversal_counters(grt_ctx *ctx, unsigned long long *counters_dev);

/* Waits for `stream` (at most timeout_ms milliseconds; 0 = no limit) and returns the first
 * error flagged by a kernel since the previous check. When the limit passes, it raises the
 * abort request (grt_abort), waits for the work in flight to stop, clears the request and
 * returns GRT_ERR_TIMEOUT: the context stays usable, the outputs of the aborted launches are
 * incomplete. A request raised by grt_abort is cleared once the stream has finished, and the
 * result is then GRT_ERR_ABORTED. */
grt_status grt_check(grt_ctx *ctx, grt_stream_t stream, uint32_t timeout_ms);

/* Asks the context's kernels to stop: a running persistent kernel (the persistent tracers, the
 * fused path tracer, scene sets, fused direct lighting) takes no further rays, paths or pixels
 * (those in flight finish), and persistent launches that start later do nothing, until
 * grt_check clears the request; one-thread-per-ray launches run to the end, each bounded by its
 * ray count. The request is a pair of copy-engine writes on a stream of its own, so it reaches
 * kernels that are running and costs them nothing while it is not raised; grt_abort may be
 * called from another host thread while the context's owner waits in grt_check. The reference
 * has no way to stop a launch (its error path resets the device,
 * rt/cuda/cuda-helpers.cpp:5-12). */
grt_status grt_abort(grt_ctx *ctx);

/* ---- ray generation steps around the traversal ---------------------------------------- */

/* Stable compaction of the valid hits (t != FLT_MAX) of n hit records: indices_dev receives
 * their ray indices in increasing order and *count_dev their number. */
grt_status grt_compact_hits(grt_ctx *ctx, const grt_hit *hits_dev, uint32_t n, uint32_t *indices_dev,
                            uint32_t *count_dev, grt_stream_t stream);

/* Allocation-free variant of grt_compact_hits. It has no counterpart in the reference; it is
 * for callers that cannot call cudaMalloc: a renderer that reserves its whole device-memory
 * budget up front and hands out memory only from its own pool, or a frame loop that cannot
 * afford cudaMalloc's implicit device synchronisation in the middle of a frame. It needs no
 * context, and its only temporary storage (one count per 2048-hit tile) is a fixed 64 KiB
 * array in device memory that every GPU loading this library holds until the process exits.
 * Limits:
 *   - n at most GRT_COMPACT_STATIC_MAX_HITS; larger n returns GRT_ERR_TOO_LARGE, nothing runs;
 *   - all calls share that one array, so calls whose kernels overlap on a GPU (for example on
 *     two streams at once) race and give wrong results: order them on one stream;
 *   - the first call on each device looks up the array's device address
 *     (cudaGetSymbolAddress) with that device current and keeps it for the life of the
 *     process; make that first call before any stream capture begins, and make no call on a
 *     device after resetting it (cudaDeviceReset).
 * The array keeps the last call's tile counts; every call overwrites the counts it reads. */
#define GRT_COMPACT_STATIC_MAX_HITS 33554432u
grt_status grt_compact_hits_static(const grt_hit *hits_dev, uint32_t n, uint32_t *indices_dev, uint32_t *count_dev,
                                   grt_stream_t stream);

/* One shadow ray per valid hit, in ray order (the any-hit rays of the reference's direct
 * lighting, gi/direct.cpp:499-534 with rt/cuda/bounce.cu:194-196): origin = hit point moved by
 * eps along the geometric normal facing the incoming ray, direction towards `light`,
 * t_min = eps, t_max = distance - eps (ray::length_exclusive, libgi/rt.h:30). shadow_rays_dev
 * needs room for n rays; *count_dev receives the number written. */
grt_status grt_shadow_rays(grt_ctx *ctx, const float *rays_dev, const grt_hit *hits_dev, uint32_t n,
                           const float light[3], float eps, float *shadow_rays_dev, uint32_t *count_dev,
                           grt_stream_t stream);

/* One grey albedo per material id (the material id is the w of each triangle); ids without
 * an entry use 0.8. n = 0 clears the table. */
grt_status grt_set_materials(grt_ctx *ctx, const float *albedo, uint32_t n);

/* ---- diffuse multi-bounce path tracing ------------------------------------------------ */

enum { GRT_PT_WAVEFRONT = 0, GRT_PT_FUSED = 1 };

typedef struct grt_pt_params {
    uint32_t max_bounces; /* bounce rays per path, default 5 */
    uint32_t rr_start;    /* Russian roulette decides before bounce rays rr_start, rr_start+1, ... (3) */
    float rr_continue;    /* survival probability of the roulette (0.8); survivors are reweighted */
    float eps;            /* origin offset along the normal and t_min of bounce rays (1e-4) */
    uint64_t seed;        /* path p draws from PCG32 stream seed + p */
    int mode;             /* GRT_PT_WAVEFRONT (one kernel per bounce) or GRT_PT_FUSED (persistent) */
    int use_graph;        /* capture the step once and replay it as a CUDA graph (stream must not be NULL) */
} grt_pt_params;

/* Result of one path: radiance = product of albedos (and roulette weights) times the sky
 * 0.5 + 0.5 d.y if the path escaped, else 0; bounces = bounce rays traced; last_ref = last hit
 * triangle (0xFFFFFFFF if none); digest = FNV-1a over (ref, t bits) of every bounce hit and a
 * 0xFFFFFFFF word for the escape. */
typedef struct grt_path_result {
    float radiance;
    uint32_t bounces;
    uint32_t last_ref;
    uint32_t digest;
} grt_path_result;

void grt_pt_params_default(grt_pt_params *params);

/* Traces n_paths diffuse paths. Path p starts at the valid primary hit number (p mod H) in ray
 * order, H being the number of valid hits among prim_hits_dev (n_primary records for the rays
 * prim_rays_dev). Each bounce samples a cosine-weighted direction around the facing geometric
 * normal (k::sample_cos_dir, rt/cuda/bounce.cu:91-142, with libgi/sampling.h:32-36 and
 * libgi/util.h:212-232), from an origin moved eps along that normal. results_dev receives
 * n_paths records; bounce_hits_dev (optional) n_paths * max_bounces closest-hit records, the
 * slots after a path's last bounce zeroed. Both modes give identical results. */
grt_status grt_pathtrace(grt_ctx *ctx, const grt_pt_params *params, const float *prim_rays_dev,
                         const grt_hit *prim_hits_dev, uint32_t n_primary, uint32_t n_paths,
                         grt_path_result *results_dev, grt_hit *bounce_hits_dev, grt_stream_t stream);

/* ---- many scenes, uneven ray batches, one launch --------------------------------------- */

/* One mesh of a scene set: host arrays in the layouts of grt_build. */
typedef struct grt_mesh {
    const float *vpos4;
    uint32_t nv;
    const uint32_t *tris4;
    uint32_t nt;
} grt_mesh;

/* Builds `count` independent scenes (the reference builder, in parallel over scenes) into
 * pooled device arrays; scene i is addressed by its index in `meshes`. Replaces any previous
 * scene set; independent of the scene of grt_build. */
grt_status grt_build_scenes(grt_ctx *ctx, const grt_mesh *meshes, uint32_t count, const grt_bvh_opts *opts);
grt_status grt_scene_info(grt_ctx *ctx, uint32_t scene, grt_bvh_stats *out);
grt_status grt_export_scene_bvh(grt_ctx *ctx, uint32_t scene, uint32_t *nodes14, uint32_t *index, uint32_t *root);

/* One batch of rays against one scene of the set: DEVICE buffers as for grt_trace. */
typedef struct grt_ray_batch {
    uint32_t scene;
    uint32_t n;
    const float *rays_dev;
    grt_hit *hits_dev;
} grt_ray_batch;

/* Traces all batches in ONE persistent launch (rays of different scenes share warps), in the
 * loop order of the selected tracer, with the results grt_trace gives per scene. The batch
 * table is a host array. Asynchronous on `stream`; batches of two calls on different streams
 * must not overlap (the context keeps one device copy of the table). */
grt_status grt_trace_multi(grt_ctx *ctx, const grt_ray_batch *batches, uint32_t count, int any_hit,
                           grt_stream_t stream);

/* ---- adjoint of the closest hit ------------------------------------------------------ */

/* Gradients of a loss through closest hits, with each ray's hit triangle held fixed. There is
 * no counterpart in the reference. For hit triangle (A, B, C) and ray (o, d) the intersection
 * (t, beta, gamma) solves the reference's Cramer system (libgi/intersect.h:36-58); the kernel
 * recomputes it from the current vertices and propagates
 *   grad_hits_dev: n x 3 floats per ray, (dL/dt, dL/dbeta, dL/dgamma)
 * back to
 *   grad_vpos_dev: 3 floats per vertex, ADDED to (zero it first), or NULL;
 *   grad_rays_dev: n x 8 floats, (dL/do xyz, 0, dL/dd xyz, 0), written, or NULL.
 * hits_dev supplies the hit triangle of each ray (misses get zero gradients); vpos_dev holds the
 * vertex positions with vstride floats per vertex (3 or 4), or is NULL for the vertices given
 * to grt_build; triangles are those given to grt_build. Vertex contributions are combined per
 * warp before the atomic adds, so the summation order (and the last bits) can vary from run to
 * run. */
grt_status grt_adjoint(grt_ctx *ctx, const float *rays_dev, const grt_hit *hits_dev, const float *grad_hits_dev,
                       uint32_t n, const float *vpos_dev, uint32_t vstride, float *grad_vpos_dev, float *grad_rays_dev,
                       grt_stream_t stream);

/* ---- direct lighting ------------------------------------------------------------------ */

/* One material: the fields of the reference's material that shading reads
 * (libgi/material.h:144-151): albedo, emission, index of refraction, roughness. */
typedef struct grt_material {
    float albedo[3];
    float emissive[3];
    float ior;
    float roughness;
} grt_material;

/* Material table of the built scene for grt_direct, indexed by the triangles' material ids
 * (ids beyond the table get the reference's default material). The lights are the triangles
 * whose material emits, chosen by power, luma(emission * area * pi), as the reference's CUDA
 * platform prepares them (rt/cuda/preprocessing.cpp:17-35). Host array, copied; must follow
 * the build; a new build drops it. */
grt_status grt_set_material_table(grt_ctx *ctx, const grt_material *materials, uint32_t n);

enum { GRT_DL_WAVEFRONT = 0, GRT_DL_FUSED = 1 };
/* The sampling strategies of the reference's direct-wf algorithm (its `sampling` setting,
 * gi/direct.cpp:503-541): a light chosen by power, or a direction on the hemisphere of the hit,
 * uniform or cosine-weighted. */
enum { GRT_DL_SAMPLE_LIGHT = 0, GRT_DL_SAMPLE_UNIFORM = 1, GRT_DL_SAMPLE_COSINE = 2 };
typedef struct grt_direct_params {
    uint32_t samples;   /* samples per pixel */
    uint32_t mode;      /* GRT_DL_WAVEFRONT or GRT_DL_FUSED */
    uint64_t seed;      /* sample s of pixel i draws from the PCG32 stream seed + s * n + i */
    uint32_t sampling;  /* GRT_DL_SAMPLE_LIGHT (0), GRT_DL_SAMPLE_UNIFORM or GRT_DL_SAMPLE_COSINE */
    uint32_t reserved;  /* must be 0 */
} grt_direct_params;

/* Direct lighting, the reference's direct-wf steps (rt/cuda/bounce.cu): for every camera ray
 * (DEVICE rays_dev, the grt_trace layout) the closest hit, then `samples` times a sample of the
 * chosen strategy and framebuffer[i] += (radiance, 1) (a hit on an emitter first adds its
 * emission and casts no ray):
 *   GRT_DL_SAMPLE_LIGHT: a light chosen by power, a point on it, an any-hit shadow ray and the
 *     light's emission (k::sample_light 210-250, k::integrate_light 380-410);
 *   GRT_DL_SAMPLE_UNIFORM / _COSINE: a direction on the hemisphere around the normal (pdf
 *     1 / 2pi, or cos / pi), a closest-hit ray and the emission of the triangle it hits
 *     (k::sample_uniform_dir 33-73, k::sample_cos_dir 91-129, k::integrate_dir 341-375);
 * each weighted by the layered GGX-coat BRDF times cos over the pdf. framebuffer_dev is n
 * float4, accumulated into. GRT_DL_WAVEFRONT runs the steps as separate launches with the
 * selected tracer; GRT_DL_FUSED runs everything in one persistent kernel in the selected
 * tracer's loop order, a warp tracing 32 pixels' rays together phase by phase. Both forms give
 * the same bits (for the speculative orders, up to the near-ties of their hits). */
grt_status grt_direct(grt_ctx *ctx, const grt_direct_params *params, const float *rays_dev, uint32_t n,
                      float *framebuffer_dev, grt_stream_t stream);

/* The shading step of the reference's primary-wf algorithm, add_hitpoint_albedo
 * (rt/cuda/kernels.cu:170-197): for every camera ray (DEVICE rays_dev) the closest hit, and
 * framebuffer[i] += (albedo of the hit triangle's material, 1), or (0, 0, 0, 1) for a miss,
 * with the materials of grt_set_material_table (untextured). mode GRT_DL_WAVEFRONT traces with
 * the selected tracer and shades in a second launch; GRT_DL_FUSED does both in one persistent
 * kernel in the selected tracer's loop order. */
grt_status grt_hit_albedo(grt_ctx *ctx, uint32_t mode, const float *rays_dev, uint32_t n, float *framebuffer_dev,
                          grt_stream_t stream);

/* ---- alpha-aware tracing ---------------------------------------------------------------- */

/* One single-channel texture: width x height alpha values, row by row. */
typedef struct grt_alpha_texture {
    uint32_t width, height;
    const float *alpha;
} grt_alpha_texture;

/* Texture data of the alpha-aware tracers, the "<tracer>-alpha" names (the reference registers
 * an alpha variant of each tracer, rt/cuda/platform.cpp:34-51). With one of them selected, a
 * triangle hit counts only where the alpha of its material's texture at the hit's interpolated
 * texture coordinate is > 0.5, as in the reference CPU tracer (rt/cpu/bvh2.cpp:109-117, 168-174;
 * libgi/rt.cpp:7-14, 32-36; nearest texel with wrap-around, libgi/scene.h:28-36). Host arrays,
 * copied: texcoords2 (2 floats per vertex of the built scene, nv = its vertex count),
 * material_texture (per material id: a texture index, or -1 for an opaque material), textures.
 * Triangles whose material id is beyond the table are opaque. Applies to grt_trace,
 * grt_trace_host and grt_pathtrace (not to scene sets); a new build drops it; a NULL
 * material_texture clears it. */
grt_status grt_set_alpha(grt_ctx *ctx, const float *texcoords2, uint32_t nv, const int32_t *material_texture,
                         uint32_t n_materials, const grt_alpha_texture *textures, uint32_t n_textures);

/* ---- BVH construction on the GPU ----------------------------------------------------- */

/* Builds the scene of grt_build on the GPU from DEVICE arrays in the same layouts (vertices
 * float4, triangles uint4 with the material id in w). No counterpart in the reference, whose
 * builds all run on the host (batch_rt::build, rt/cuda/base.cpp:88-117): a binary tree over the
 * triangles (see grt_set_device_builder), subtrees of at most max_tris_per_node (1..16)
 * triangles turned into leaves (by the SAH builder always, as the reference's builder does; by
 * the others where the SAH cost says so), and its 4-wide collapse.
 * The tree differs from the reference builder's, so closest hits equal the reference's except
 * near-ties (any-hit answers are equal). Every tracer can trace it; grt_export_bvh has no
 * reference tree to export and fails. The arrays are copied, so the caller may free them after
 * the call. Ordered after earlier work on `stream`; returns when the build is done. At most
 * 2^27 - 1 triangles. */
grt_status grt_build_device(grt_ctx *ctx, const float *vpos4_dev, uint32_t nv, const uint32_t *tris4_dev,
                            uint32_t nt, uint32_t max_tris_per_node, grt_stream_t stream);

/* grt_build_scenes with the GPU builder: the vpos4 / tris4 pointers of `meshes` (a host array)
 * are DEVICE pointers, read during the call only. grt_export_scene_bvh fails for such a set. */
grt_status grt_build_scenes_device(grt_ctx *ctx, const grt_mesh *meshes, uint32_t count, uint32_t max_tris_per_node,
                                   grt_stream_t stream);

/* How the GPU builder forms the binary tree:
 *   GRT_DEVICE_BUILD_SAH: top-down splits with the reference builder's SAH rule
 *     (rt/cpu/bvh-ctor.h:386-488: the major axis of each node's box, evenly spaced candidate
 *     planes, see grt_set_device_sah_planes, the least surface-area cost), the candidates binned
 *     on the GPU instead of partitioned in place. Trees of the host SAH builder's quality; the
 *     top part of the tree takes a few launches per level;
 *   GRT_DEVICE_BUILD_PLOC: agglomerative clustering (PLOC, Meister and Bittner 2018) in Morton
 *     order: clusters merge with their mutual nearest neighbour (smallest union surface area)
 *     among the 16 on either side in the list, iteration after iteration;
 *   GRT_DEVICE_BUILD_LBVH: the radix tree of the Morton codes (Karras 2012), built in one pass:
 *     the fastest build (for scenes rebuilt every frame), trees that trace a few per cent slower.
 * GRT_DEVICE_BUILD_DEFAULT is GRT_DEVICE_BUILD_SAH. grt_build_scenes_device builds the scenes of
 * a set concurrently (up to 8 host threads, each with a stream of its own); with the SAH method
 * the trees of all its scenes are built together, level by level over all their triangles,
 * each scene's tree the one it gets alone. A builder that made a malformed tree (an internal
 * fault, never an input's) fails the build with GRT_ERR_TRAVERSAL. */
enum { GRT_DEVICE_BUILD_DEFAULT = 0, GRT_DEVICE_BUILD_LBVH = 1, GRT_DEVICE_BUILD_PLOC = 2, GRT_DEVICE_BUILD_SAH = 3 };
grt_status grt_set_device_builder(grt_ctx *ctx, int method);
/* Candidate planes per node of GRT_DEVICE_BUILD_SAH (1..256, default 256; as many as a node has
 * triangles when that is fewer), the reference builder's `planes` option. */
grt_status grt_set_device_sah_planes(grt_ctx *ctx, uint32_t planes);

/* Refits the context's scene (built by grt_build or grt_build_device) to new vertex positions:
 * DEVICE float4 array of the built scene's nv vertices, copied. The tree keeps its topology;
 * the triangle records and every node box (binary and 4-wide) are recomputed on the GPU from
 * the new positions, which is far cheaper than a build when the mesh changes a little between
 * uses (the steps of a gradient descent on the vertices). No counterpart in the reference,
 * which rebuilds on every change (batch_rt::build, rt/cuda/base.cpp:88-117). The refitted tree
 * is no longer the reference builder's: closest hits equal the reference's on the new vertices
 * except near-ties, and grt_export_bvh fails until the next build. Ordered after earlier work on
 * `stream`; returns when the refit is done. */
grt_status grt_refit(grt_ctx *ctx, const float *vpos4_dev, uint32_t nv, grt_stream_t stream);

/* ---- timing ----------------------------------------------------------------------------- */

/* Per-call device times, the counterpart of the reference's wavefront step timers
 * (time_this_wf_step, libgi/wavefront-rt.h:29: a CUDA event pair per step, folded into its
 * stats timer, rt/cuda/base.cpp:17-45). While enabled, every call below of the given kind
 * records an event pair on its stream around its launches (not while the stream is being
 * captured into a graph); grt_timing_stats waits for the recorded pairs and returns, per kind,
 * the number of calls and their summed device time since the last reset. Off by default: the
 * traversal calls then record nothing. */
enum {
    GRT_TIME_TRACE = 0,        /* grt_trace */
    GRT_TIME_TRACE_MULTI = 1,  /* grt_trace_multi */
    GRT_TIME_PATHTRACE = 2,    /* grt_pathtrace */
    GRT_TIME_DIRECT = 3,       /* grt_direct, grt_hit_albedo */
    GRT_TIME_ADJOINT = 4,      /* grt_adjoint */
    GRT_TIME_TREE = 5,         /* grt_build_device, grt_build_scenes_device, grt_refit */
    GRT_TIME_RAYS = 6,         /* grt_incoherent_rays, grt_camera_rays, grt_compact_hits, grt_shadow_rays */
    GRT_TIME_KINDS = 7
};
typedef struct grt_timing {
    uint64_t calls[GRT_TIME_KINDS];
    double ms[GRT_TIME_KINDS];
} grt_timing;
grt_status grt_set_timing(grt_ctx *ctx, int enabled);
/* Synchronises with the recorded calls; `reset` != 0 starts the totals again afterwards. */
grt_status grt_timing_stats(grt_ctx *ctx, grt_timing *out, int reset);

/* ---- ray generation ------------------------------------------------------------------- */

/* The incoherent test rays of the reference CUDA tracer's `incoherence r1 r2` setting
 * (rt/cuda/base.cpp:120-133; batch_cam_ray_setup, rt/cuda/rni.cpp:36-84; setup_ray_incoherent,
 * rt/cuda/kernels.cu:75-156), written to DEVICE rays_dev (n rays, the grt_trace layout): two
 * balls at the quarter points of the largest dimension of the built scene's vertex extent,
 * radius r_max = a quarter of that dimension; each ray starts at a uniform point in the ball of
 * radius r1 * r_max around the first centre and aims at a uniform point in the ball of radius
 * r2 * r_max around the second (a radius of 0: the centre), t_min 0, t_max FLT_MAX. The random
 * numbers come from a PCG32 stream per ray (seed + ray index) instead of cuRAND's MTGP32. */
grt_status grt_incoherent_rays(grt_ctx *ctx, float r1, float r2, uint64_t seed, float *rays_dev, uint32_t n,
                               grt_stream_t stream);

/* A pinhole camera as the reference's struct camera holds it (libgi/camera.h:7-24): position,
 * view direction (normalised), up vector, and the half extents of the near plane at distance 1
 * (camera::update_frustum: near_h = tan(fovy / 2), near_w = aspect * near_h). */
typedef struct grt_camera {
    float pos[3], dir[3], up[3];
    float near_w, near_h;
} grt_camera;

/* The camera rays of a w x h image on the device: the primary-ray step of the wavefront
 * algorithms (batch_cam_ray_setup -> setup_rays, rt/cuda/rni.cpp:86-99, rt/cuda/kernels.cu:26-61)
 * computed as the reference's cam_ray computes them on the CPU (libgi/camera.cpp:11-28), bit for
 * bit: U = normalize(cross(dir, up)), V = normalize(cross(U, dir)),
 * u = near_w ((x + 0.5 + offset.x) / w * 2 - 1), v likewise with y and near_h,
 * d = normalize(dir + U u + V v); origin pos, t_min = 1e-4 (ray::eps), t_max = FLT_MAX. Ray (x, y)
 * goes to index y w + x of DEVICE rays_dev (the grt_trace layout, 2 w h float4).
 * Sub-pixel offsets (cam_ray's `offset`, in [-0.5, 0.5)): offsets_dev, two floats per pixel in
 * device memory, when given; otherwise with jitter != 0 two uniform_float draws minus 0.5 from a
 * PCG32 stream per pixel (rng_pcg::set_sequence(seed + pixel index)); otherwise the pixel
 * centres. (The reference's CUDA setup_rays builds rays with unnormalised U and V and t_min 0;
 * this step follows cam_ray, the rays of the CPU tracer the hits are defined against.) */
grt_status grt_camera_rays(grt_ctx *ctx, const grt_camera *camera, uint32_t w, uint32_t h, const float *offsets_dev,
                           int jitter, uint64_t seed, float *rays_dev, grt_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* GRT_H */
