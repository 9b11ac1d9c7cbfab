// One persistent launch over many scenes and uneven ray batches.
//
// The reference traces one scene per platform (wf::cuda::batch_rt, rt/cuda/base.h:403-429); a
// batch of many small and large scenes would take one launch per scene, each with its own
// tail. Here every batch (scene index, ray count, ray and hit buffers) gets a range of a global
// ray index; persistent warps take rays from one counter, and each lane finds its batch by a
// binary search over the batch offsets, then traverses with that batch's scene descriptor.
// Lanes of one warp may work on different scenes at the same time.
#include "multi.hpp"
#include "traverse.cuh"

namespace grt {

namespace {

constexpr unsigned kFull = 0xffffffffu;

// index of the last batch whose offset is <= g (offsets ascending, offsets[0] = 0)
__device__ __forceinline__ uint32_t find_batch(const multi_batch *__restrict__ b, uint32_t nb, uint32_t g) {
    uint32_t lo = 0, hi = nb;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(&b[mid].offset) <= g)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

template <int ORDER, bool ANY, int FP = 0>
__global__ void __launch_bounds__(256) k_trace_multi(const dev_scene *__restrict__ scenes,
                                                     const multi_batch *__restrict__ batches, uint32_t nbatch,
                                                     uint32_t total, unsigned *err, unsigned *counter,
                                                     int refill_threshold, int refill_period, int cap,
                                                     spec_cfg spec) {
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
    dev_scene sc{};
    grt_hit *hits = nullptr;
    uint32_t idx = 0;
    bool have = false, plain = false, exhausted = false;
    for (;;) {
        if (!exhausted) {
            const unsigned need = __ballot_sync(kFull, !have);
            if (need) {
                const unsigned cnt = __popc(need);
                unsigned base = 0;
                if (lane == 0) base = atomicAdd(counter, cnt);
                base = __shfl_sync(kFull, base, 0);
                if (base + cnt >= total) exhausted = true;
                if (!have) {
                    const uint32_t g = base + __popc(need & lanes_below);
                    if (g < total) {
                        const uint32_t b = find_batch(batches, nbatch, g);
                        const multi_batch mb = batches[b];
                        idx = g - mb.offset;
                        sc = scenes[mb.scene];
                        hits = mb.hits;
                        r = load_ray(mb.rays, idx);
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
        for (int it = 1;; ++it) {
            if (SPEC)
                trav_spec_iter<ANY, false, WIDE, false, kFastVisits[FP], kFastPend[FP]>(s, have, plain, sc, r, stk,
                                                                                        stride, cap, spec, err);
            else if (have && plain)
                trav_advance<ORDER, ANY, false, true>(s, sc, r, stk, stride, cap, err);
            else if (have)
                trav_advance<ORDER, ANY, false, false>(s, sc, r, stk, stride, cap, err);
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

using multi_fn = void (*)(const dev_scene *, const multi_batch *, uint32_t, uint32_t, unsigned *, unsigned *, int, int,
                          int, spec_cfg);

// The scene-set kernel instance for fast-path instance `fp` (speculative order only).
template <int ORDER, bool ANY> multi_fn multi_kernel_of(int fp) {
    if (ORDER == SPECULATIVE) {
        switch (fp) {
            case 1: return k_trace_multi<ORDER, ANY, ORDER == SPECULATIVE ? 1 : 0>;
            case 2: return k_trace_multi<ORDER, ANY, ORDER == SPECULATIVE ? 2 : 0>;
            case 3: return k_trace_multi<ORDER, ANY, ORDER == SPECULATIVE ? 3 : 0>;
            case 4: return k_trace_multi<ORDER, ANY, ORDER == SPECULATIVE ? 4 : 0>;
            default: break;
        }
    }
    return k_trace_multi<ORDER, ANY>;
}

template <int ORDER, bool ANY>
cudaError_t multi_launch(const dev_scene *scenes, const multi_batch *batches, uint32_t nbatch, uint32_t total,
                         const launch_params &lp, unsigned *err, unsigned *counter, cudaStream_t st) {
    const size_t smem = (size_t)lp.stack_entries * lp.block_threads * sizeof(int);
    cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(unsigned), st);
    if (e != cudaSuccess) return e;
    multi_kernel_of<ORDER, ANY>(fast_path_of(lp.spec))<<<lp.grid_blocks, lp.block_threads, smem, st>>>(
        scenes, batches, nbatch, total, err, counter, lp.refill_threshold, lp.refill_period, lp.stack_entries, lp.spec);
    return cudaGetLastError();
}

template <int ORDER>
cudaError_t multi_any(bool any_hit, const dev_scene *scenes, const multi_batch *batches, uint32_t nbatch,
                      uint32_t total, const launch_params &lp, unsigned *err, unsigned *counter, cudaStream_t st) {
    return any_hit ? multi_launch<ORDER, true>(scenes, batches, nbatch, total, lp, err, counter, st)
                   : multi_launch<ORDER, false>(scenes, batches, nbatch, total, lp, err, counter, st);
}

template <int ORDER> cudaError_t attrs(int bytes) {
    const cudaFuncAttribute a = cudaFuncAttributeMaxDynamicSharedMemorySize;
    cudaError_t e = cudaSuccess;
    for (int fp = 0; fp < kFastPaths && e == cudaSuccess; ++fp) {
        e = cudaFuncSetAttribute(multi_kernel_of<ORDER, false>(fp), a, bytes);
        if (e == cudaSuccess) e = cudaFuncSetAttribute(multi_kernel_of<ORDER, true>(fp), a, bytes);
    }
    return e;
}

}  // namespace

cudaError_t launch_trace_multi(const dev_scene *scenes, const multi_batch *batches, uint32_t nbatch, uint32_t total,
                               bool any_hit, const launch_params &lp, unsigned *err, unsigned *counter,
                               cudaStream_t st) {
    if (total == 0) return cudaSuccess;
    if (!spec_ok(lp.spec)) return cudaErrorInvalidValue;
    switch (lp.order) {
        case WHILE_WHILE: return multi_any<WHILE_WHILE>(any_hit, scenes, batches, nbatch, total, lp, err, counter, st);
        case SPECULATIVE: return multi_any<SPECULATIVE>(any_hit, scenes, batches, nbatch, total, lp, err, counter, st);
        case WIDE_SPECULATIVE:
            return multi_any<WIDE_SPECULATIVE>(any_hit, scenes, batches, nbatch, total, lp, err, counter, st);
        default: return multi_any<IF_IF>(any_hit, scenes, batches, nbatch, total, lp, err, counter, st);
    }
}

cudaError_t prepare_multi_kernels() {
    const int bytes = kStackLarge * 256 * (int)sizeof(int);
    cudaError_t e = attrs<IF_IF>(bytes);
    if (e == cudaSuccess) e = attrs<WHILE_WHILE>(bytes);
    if (e == cudaSuccess) e = attrs<SPECULATIVE>(bytes);
    if (e == cudaSuccess) e = attrs<WIDE_SPECULATIVE>(bytes);
    return e;
}

int multi_blocks_per_sm(int block_threads, int stack_entries, int order, const spec_cfg &spec) {
    int blocks = 0;
    const size_t smem = (size_t)stack_entries * block_threads * sizeof(int);
    const int fp = fast_path_of(spec);
    const void *fn = order == WHILE_WHILE        ? (const void *)multi_kernel_of<WHILE_WHILE, false>(fp)
                     : order == SPECULATIVE      ? (const void *)multi_kernel_of<SPECULATIVE, false>(fp)
                     : order == WIDE_SPECULATIVE ? (const void *)multi_kernel_of<WIDE_SPECULATIVE, false>(fp)
                                                 : (const void *)multi_kernel_of<IF_IF, false>(fp);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, fn, block_threads, smem) != cudaSuccess) return 1;
    return blocks > 0 ? blocks : 1;
}

}  // namespace grt
