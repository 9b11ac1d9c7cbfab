// Closest-hit / any-hit traversal kernels for sm_103a.
//
// Two kernel shapes replace the reference's CUDA variants (rt/cuda/trace-kernels.cu), each in
// the if-if, while-while and speculative while-while loop orders (traverse.cuh):
//   * k_trace_plain — one thread per ray, the wavefront baseline (the role of ifif_trace and
//     whilewhile_trace, rt/cuda/trace-kernels.cu:238-316);
//   * k_trace_persistent — persistent warps that refill lanes whose ray finished from a global
//     ray counter whenever fewer than `refill_threshold` lanes are still busy (the idea of
//     dynamicwhilewhile_trace, rt/cuda/trace-kernels.cu:702-876, restructured so that every
//     ballot is taken by all 32 lanes at a uniform point of the loop, and the counter is reset
//     by the host before the launch instead of by the kernel's own threads).
// In the if-if and while-while orders every ray visits its nodes in the reference's order, so
// results are identical to the reference CPU tracer; the speculative order may differ from it
// in near-ties only.
#include "traverse.cuh"

namespace grt {

namespace {

constexpr unsigned kFull = 0xffffffffu;

// Resident blocks of 256 threads asked of the compiler per loop order, as measured on GB300
// (plain bounce traces of the sphere scene): left to itself the compiler holds the speculative
// loop to 48 registers and spills; at 4 blocks (64 registers at most) the while-while and
// speculative loops run 4 % / 1 % faster, the if-if loop is fastest at 5 and the 4-wide loop
// with no bound (72 registers).
template <int ORDER>
constexpr int plain_min_blocks() {
    return ORDER == IF_IF ? 5 : ORDER == WIDE_SPECULATIVE ? 1 : 4;
}

template <int ORDER, bool ANY, bool COUNT, bool ALPHA, int FP = 0>
__global__ void __launch_bounds__(256, plain_min_blocks<ORDER>()) k_trace_plain(const float4 *__restrict__ rays, grt_hit *__restrict__ hits,
                                                     uint32_t n, const uint32_t *__restrict__ n_dev, dev_scene sc,
                                                     unsigned *err, unsigned long long *counters, int cap,
                                                     spec_cfg spec) {
    extern __shared__ int s_stack[];
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (n_dev) n = *n_dev;  // ray count produced on the device (wavefront queues)
    const bool active = i < n;
    constexpr bool SPEC = ORDER == SPECULATIVE || ORDER == WIDE_SPECULATIVE;
    constexpr bool WIDE = ORDER == WIDE_SPECULATIVE;
    if (!SPEC && !active) return;
    ray_t r = {};
    if (active) r = load_ray(rays, i);
    trav_t s;
    trav_init(s, sc, r, WIDE);
    int *stk = s_stack + threadIdx.x;
    const int stride = blockDim.x;
    const bool plain = active && sc.finite && ray_is_plain(r);
    if (SPEC) {  // the whole warp stays in the loop until its last ray ends
        while (__any_sync(kFull, active && !s.done))
            trav_spec_iter<ANY, COUNT, WIDE, ALPHA, kFastVisits[FP], kFastPend[FP]>(s, active, plain, sc, r, stk,
                                                                                      stride, cap, spec, err);
        if (!active) return;
    } else if (plain) {  // one loop per slab variant: the choice is made once per ray
        while (!s.done) trav_advance<ORDER, ANY, COUNT, true, ALPHA>(s, sc, r, stk, stride, cap, err);
    } else {
        while (!s.done) trav_advance<ORDER, ANY, COUNT, false, ALPHA>(s, sc, r, stk, stride, cap, err);
    }
    store_hit<ANY>(hits, i, s);
    if (COUNT) {
        atomicAdd(counters + 0, 1ull);
        atomicAdd(counters + 1, (unsigned long long)s.n_inner);
        atomicAdd(counters + 2, (unsigned long long)s.n_tri);
    }
}

template <int ORDER, bool ANY, bool ALPHA, int FP = 0>
__global__ void __launch_bounds__(256) k_trace_persistent(const float4 *__restrict__ rays, grt_hit *__restrict__ hits,
                                                          uint32_t n, dev_scene sc, unsigned *err,
                                                          unsigned *counter, int refill_threshold, int refill_period,
                                                          int cap, spec_cfg spec) {
    extern __shared__ int s_stack[];
    if (stop_requested_at_entry(err)) return;  // the host asked the context to stop
    constexpr bool SPEC = ORDER == SPECULATIVE || ORDER == WIDE_SPECULATIVE;
    constexpr bool WIDE = ORDER == WIDE_SPECULATIVE;
    const unsigned lane = threadIdx.x & 31u;
    const unsigned lanes_below = (1u << lane) - 1u;
    int *stk = s_stack + threadIdx.x;
    const int stride = blockDim.x;
    trav_t s;
    ray_t r;
    uint32_t idx = 0;
    bool have = false, plain = false, exhausted = false;
    for (;;) {
        // refill the lanes without a ray (all 32 lanes arrive here together)
        if (!exhausted) {
            const unsigned need = __ballot_sync(kFull, !have);
            if (need) {
                const unsigned cnt = __popc(need);
                unsigned base = 0;
                if (lane == 0) base = atomicAdd(counter, cnt);
                base = __shfl_sync(kFull, base, 0);
                if (base + cnt >= n) exhausted = true;
                if (!have) {
                    const uint32_t my = base + __popc(need & lanes_below);
                    if (my < n) {
                        idx = my;
                        r = load_ray(rays, my);
                        trav_init(s, sc, r, WIDE);
                        plain = sc.finite && ray_is_plain(r);
                        have = true;
                        if (s.done) {  // empty scene
                            store_hit<ANY>(hits, idx, s);
                            have = false;
                        }
                    }
                }
            }
        }
        if (__ballot_sync(kFull, have) == 0) {
            if (exhausted) break;
            continue;
        }
        // traverse; every `refill_period` iterations the warp counts its busy lanes
        for (int it = 1;; ++it) {
            if (SPEC)
                trav_spec_iter<ANY, false, WIDE, ALPHA, kFastVisits[FP], kFastPend[FP]>(s, have, plain, sc, r, stk,
                                                                                        stride, cap, spec, err);
            else if (have && plain)
                trav_advance<ORDER, ANY, false, true, ALPHA>(s, sc, r, stk, stride, cap, err);
            else if (have)
                trav_advance<ORDER, ANY, false, false, ALPHA>(s, sc, r, stk, stride, cap, err);
            if (have && s.done) {
                store_hit<ANY>(hits, idx, s);
                have = false;
            }
            if (it % refill_period == 0) {
                const int busy = __popc(__ballot_sync(kFull, have));
                if (busy == 0 || (!exhausted && busy < refill_threshold)) break;
            }
        }
    }
}

template <int ORDER, bool ANY>
cudaError_t plain_launch(const dev_scene &sc, const float4 *rays, grt_hit *hits, uint32_t n, const uint32_t *n_dev,
                         const launch_params &lp, unsigned *err, cudaStream_t st) {
    const int bt = lp.block_threads;
    const unsigned blocks = (n + bt - 1) / bt;
    const size_t smem = (size_t)lp.stack_entries * bt * sizeof(int);
    const int cap = lp.stack_entries;
    if (lp.counters && sc.alpha)
        k_trace_plain<ORDER, ANY, true, true><<<blocks, bt, smem, st>>>(rays, hits, n, n_dev, sc, err, lp.counters, cap,
                                                                        lp.spec);
    else if (lp.counters)
        k_trace_plain<ORDER, ANY, true, false><<<blocks, bt, smem, st>>>(rays, hits, n, n_dev, sc, err, lp.counters, cap,
                                                                         lp.spec);
    else if (sc.alpha)
        k_trace_plain<ORDER, ANY, false, true><<<blocks, bt, smem, st>>>(rays, hits, n, n_dev, sc, err, nullptr, cap,
                                                                         lp.spec);
    else if (ORDER == SPECULATIVE && fast_path_of(lp.spec) == 3)  // the one-thread-per-ray default
        k_trace_plain<ORDER, ANY, false, false, ORDER == SPECULATIVE ? 3 : 0><<<blocks, bt, smem, st>>>(
            rays, hits, n, n_dev, sc, err, nullptr, cap, lp.spec);
    else
        k_trace_plain<ORDER, ANY, false, false><<<blocks, bt, smem, st>>>(rays, hits, n, n_dev, sc, err, nullptr, cap,
                                                                          lp.spec);
    return cudaGetLastError();
}

// The persistent kernel instance for alpha-aware tracing or fast-path instance `fp` (the
// speculative order only has instances beyond 0).
using persistent_fn = void (*)(const float4 *, grt_hit *, uint32_t, dev_scene, unsigned *, unsigned *, int, int, int,
                               spec_cfg);
template <int ORDER, bool ANY> persistent_fn persistent_kernel_of(bool alpha, int fp) {
    if (alpha) return k_trace_persistent<ORDER, ANY, true>;
    if (ORDER == SPECULATIVE) {
        switch (fp) {
            case 1: return k_trace_persistent<ORDER, ANY, false, ORDER == SPECULATIVE ? 1 : 0>;
            case 2: return k_trace_persistent<ORDER, ANY, false, ORDER == SPECULATIVE ? 2 : 0>;
            case 3: return k_trace_persistent<ORDER, ANY, false, ORDER == SPECULATIVE ? 3 : 0>;
            case 4: return k_trace_persistent<ORDER, ANY, false, ORDER == SPECULATIVE ? 4 : 0>;
            default: break;
        }
    }
    return k_trace_persistent<ORDER, ANY, false>;
}

template <int ORDER, bool ANY>
cudaError_t persistent_launch(const dev_scene &sc, const float4 *rays, grt_hit *hits, uint32_t n,
                              const launch_params &lp, unsigned *err, unsigned *counter, cudaStream_t st) {
    const int bt = lp.block_threads;
    const size_t smem = (size_t)lp.stack_entries * bt * sizeof(int);
    cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(unsigned), st);
    if (e != cudaSuccess) return e;
    const int fp = (ORDER == SPECULATIVE && !sc.alpha) ? fast_path_of(lp.spec) : 0;
    persistent_kernel_of<ORDER, ANY>(sc.alpha != nullptr, fp)<<<lp.grid_blocks, bt, smem, st>>>(
        rays, hits, n, sc, err, counter, lp.refill_threshold, lp.refill_period, lp.stack_entries, lp.spec);
    return cudaGetLastError();
}

// Dispatch of the runtime choices (loop order, any-hit) to template instances.
template <template <int, bool> class F, typename... A>
cudaError_t dispatch(int order, bool any_hit, A &&...a) {
    if (order == WIDE_SPECULATIVE)
        return any_hit ? F<WIDE_SPECULATIVE, true>::run(a...) : F<WIDE_SPECULATIVE, false>::run(a...);
    if (order == SPECULATIVE) return any_hit ? F<SPECULATIVE, true>::run(a...) : F<SPECULATIVE, false>::run(a...);
    if (order == WHILE_WHILE) return any_hit ? F<WHILE_WHILE, true>::run(a...) : F<WHILE_WHILE, false>::run(a...);
    return any_hit ? F<IF_IF, true>::run(a...) : F<IF_IF, false>::run(a...);
}

template <int O, bool A> struct plain_f {
    template <typename... X> static cudaError_t run(X &&...x) { return plain_launch<O, A>(x...); }
};
template <int O, bool A> struct persistent_f {
    template <typename... X> static cudaError_t run(X &&...x) { return persistent_launch<O, A>(x...); }
};
template <int O, bool A> struct attr_f {
    static cudaError_t run(int bytes) {
        const cudaFuncAttribute a = cudaFuncAttributeMaxDynamicSharedMemorySize;
        cudaError_t e = cudaFuncSetAttribute(k_trace_plain<O, A, false, false>, a, bytes);
        if (e == cudaSuccess) e = cudaFuncSetAttribute(k_trace_plain<O, A, true, false>, a, bytes);
        if (e == cudaSuccess) e = cudaFuncSetAttribute(k_trace_plain<O, A, false, true>, a, bytes);
        if (e == cudaSuccess) e = cudaFuncSetAttribute(k_trace_plain<O, A, true, true>, a, bytes);
        if (e == cudaSuccess && O == SPECULATIVE)
            e = cudaFuncSetAttribute(k_trace_plain<O, A, false, false, O == SPECULATIVE ? 3 : 0>, a, bytes);
        for (int fp = 0; fp < kFastPaths && e == cudaSuccess; ++fp)
            e = cudaFuncSetAttribute(persistent_kernel_of<O, A>(false, fp), a, bytes);
        if (e == cudaSuccess) e = cudaFuncSetAttribute(persistent_kernel_of<O, A>(true, 0), a, bytes);
        return e;
    }
};
template <int O, bool A> struct occupancy_f {
    static cudaError_t run(int block_threads, int stack_entries, bool alpha, int fp, int *blocks) {
        const size_t smem = (size_t)stack_entries * block_threads * sizeof(int);
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, persistent_kernel_of<O, A>(alpha, fp),
                                                             block_threads, smem);
    }
};

}  // namespace

cudaError_t launch_trace_plain(const dev_scene &sc, const float4 *rays, grt_hit *hits, uint32_t n, bool any_hit,
                               const launch_params &lp, unsigned *err, cudaStream_t stream, const uint32_t *n_dev) {
    if (n == 0) return cudaSuccess;
    if (!spec_ok(lp.spec)) return cudaErrorInvalidValue;
    return dispatch<plain_f>(lp.order, any_hit, sc, rays, hits, n, n_dev, lp, err, stream);
}

cudaError_t launch_trace_persistent(const dev_scene &sc, const float4 *rays, grt_hit *hits, uint32_t n, bool any_hit,
                                    const launch_params &lp, unsigned *err, unsigned *counter, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    if (!spec_ok(lp.spec)) return cudaErrorInvalidValue;
    return dispatch<persistent_f>(lp.order, any_hit, sc, rays, hits, n, lp, err, counter, stream);
}

cudaError_t prepare_trace_kernels() {
    const int bytes = kStackLarge * 256 * (int)sizeof(int);  // largest stack at 256 threads
    for (int order : {(int)IF_IF, (int)WHILE_WHILE, (int)SPECULATIVE, (int)WIDE_SPECULATIVE})
        for (bool any : {false, true}) {
            cudaError_t e = dispatch<attr_f>(order, any, bytes);
            if (e != cudaSuccess) return e;
        }
    return cudaSuccess;
}

int persistent_blocks_per_sm(int block_threads, int stack_entries, bool any_hit, int order, bool alpha,
                             const spec_cfg &spec) {
    int blocks = 0;
    const int fp = (order == SPECULATIVE && !alpha) ? fast_path_of(spec) : 0;
    if (dispatch<occupancy_f>(order, any_hit, block_threads, stack_entries, alpha, fp, &blocks) != cudaSuccess) return 1;
    return blocks > 0 ? blocks : 1;
}

}  // namespace grt
