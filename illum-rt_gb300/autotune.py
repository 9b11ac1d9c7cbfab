"""Autotuner for the persistent kernels: loop order, warps per block, refill threshold and
period, the tree (leaf size, SAH candidate planes, early split clipping), and for the
speculative order its warp-level parameters (leaves postponed per lane, lanes still searching
when the warp leaves its node phase, node visits per warp vote) and the traversal stack size.

For every candidate it builds the scene's BVH with the reference builder's options
(`max_triangles_per_node`, `number_of_planes`, `esc`), sets the launch parameters through
grt_set_tuning and times the fused path-tracing step (persistent primary trace + fused bounce
loop) with CUDA events. Three stages: launch parameters and leaf size on trees of the
reference's 16 planes with clipping; then, with the best launch, every leaf size, plane count
and clipping choice; then the launch parameters again on the best tree; then, for a speculative
tracer, the grid of its warp-level parameters and stack sizes on that tree. The fastest
configuration is written to tuning.json under "<GPU name>|<scene class>", where bench.py picks
it up. Results do not depend on the launch parameters; other tree options give a different
(equally reference-built) BVH.

With --workload soups64 it tunes the scene-set trace instead: the 64 uneven soups of the
benchmark, GPU-built trees of each leaf size, one persistent launch over all their rays, timed
per candidate, written under "<GPU name>|soups64".

Usage: python illum-rt_gb300/autotune.py [--quick] [--paths N] [--workload spheres|soups64]
"""
from __future__ import annotations

import argparse
import itertools
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
TABLE = os.path.join(HERE, "tuning.json")


def _load_pkg():
    sys.path.insert(0, os.path.dirname(HERE))
    import __graft_entry__ as ge
    ge.load_package()
    from illum_rt_gb300 import api, workloads
    return api, workloads


def time_config(rt, api, rays, hits, results, n_paths, stream, reps=3) -> float:
    import torch
    p = api.BatchRayTracer.pt_params(mode=api.PT_FUSED, use_graph=0)
    best = float("inf")
    for i in range(reps + 1):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        rt.trace(rays, hits, False, stream.cuda_stream)
        rt.pathtrace(p, rays, hits, n_paths, results, None, stream.cuda_stream)
        e1.record(stream)
        e1.synchronize()
        if i:  # the first run is a warm-up
            best = min(best, e0.elapsed_time(e1))
    rt.check(stream.cuda_stream)
    return best


def tune(quick: bool = False, n_paths: int = 4 << 20, res: int = 1024, log=print) -> dict:
    import torch
    api, wl = _load_pkg()
    sc, rays_np = wl.spheres_primary(res=res)
    rays = torch.from_numpy(rays_np).cuda()
    hits = torch.zeros((rays.shape[0], 4), device="cuda")
    results = torch.zeros((n_paths, 4), dtype=torch.int32, device="cuda")
    stream = torch.cuda.Stream()
    rt = api.BatchRayTracer(0)
    orders = ["persistent-while-while"] if quick else ["persistent-while-while", "persistent-if-if",
                                                       "persistent-speculative-while-while",
                                                       "persistent-bvh4-speculative-while-while"]
    leaf_sizes = [4] if quick else [2, 3, 4, 6, 8]
    blocks = [128] if quick else [64, 128, 256]
    thresholds = [12, 20, 28] if quick else [8, 12, 16, 20, 24, 28, 32]
    periods = [1, 4] if quick else [1, 2, 4, 8]
    plane_counts = [16] if quick else [16, 32, 64, 128, 256]
    clipping = [True] if quick else [True, False]
    best = None
    searched = 0
    t0 = time.time()

    def launch_sweep(tracers, tree):
        nonlocal best, searched
        for tracer, bt, th, per in itertools.product(tracers, blocks, thresholds, periods):
            rt.select(tracer)
            rt.set_tuning(block_threads=bt, refill_threshold=th, refill_period=per, blocks_per_sm=0)
            ms = time_config(rt, api, rays, hits, results, n_paths, stream)
            cfg = {"tracer": tracer, **tree, "block_threads": bt, "refill_threshold": th, "refill_period": per,
                   "ms": ms}
            log(json.dumps(cfg))
            searched += 1
            if best is None or ms < best["ms"]:
                best = cfg

    def build(tree):
        rt.build(sc.vpos, sc.tris, max_tris=tree["max_tris"], planes=tree["planes"], esc=bool(tree["esc"]))

    # stage 1: launch parameters and leaf size on the reference's tree options
    for leaf in leaf_sizes:
        tree = {"max_tris": leaf, "planes": 16, "esc": 1}
        build(tree)
        launch_sweep(orders, tree)
    # stage 2: the tree options with the best launch
    launch = {k: best[k] for k in ("tracer", "block_threads", "refill_threshold", "refill_period")}
    rt.select(launch["tracer"])
    rt.set_tuning(block_threads=launch["block_threads"], refill_threshold=launch["refill_threshold"],
                  refill_period=launch["refill_period"], blocks_per_sm=0)
    for leaf, planes, esc in itertools.product(leaf_sizes, plane_counts, clipping):
        tree = {"max_tris": leaf, "planes": planes, "esc": int(esc)}
        if planes == 16 and esc:
            continue  # timed in stage 1
        build(tree)
        ms = time_config(rt, api, rays, hits, results, n_paths, stream)
        cfg = {**launch, **tree, "ms": ms}
        log(json.dumps(cfg))
        searched += 1
        if ms < best["ms"]:
            best = cfg
    # stage 3: the launch parameters again on the best tree
    tree = {k: best[k] for k in ("max_tris", "planes", "esc")}
    build(tree)
    if tree != {"max_tris": best["max_tris"], "planes": 16, "esc": 1}:
        launch_sweep([best["tracer"]], tree)
    # stage 4: the speculative order's warp-level parameters and the stack size
    if "speculative" in best["tracer"]:
        best = spec_sweep(rt, best, quick, log,
                          lambda: time_config(rt, api, rays, hits, results, n_paths, stream))
        searched += best.pop("_searched")
    rt.close()
    best["searched"] = searched
    best["seconds"] = round(time.time() - t0, 1)
    return best


SPEC_GRID = {"spec_pend": [1, 2, 3], "spec_exit": [4, 6, 8, 12], "spec_visits": [3, 5], "stack_entries": [0, 32]}
SPEC_GRID_QUICK = {"spec_pend": [2], "spec_exit": [8], "spec_visits": [3, 5], "stack_entries": [0]}


def spec_sweep(rt, best: dict, quick: bool, log, timer) -> dict:
    """Times every point of the speculative grid (leaves postponed, exit lanes, visits per vote,
    stack entries; 0 = the tree's depth) with the best tracer, tree and launch; returns the
    best configuration with its grid values (and the number of points under `_searched`)."""
    launch = {k: best[k] for k in ("block_threads", "refill_threshold", "refill_period")}
    grid = SPEC_GRID_QUICK if quick else SPEC_GRID
    keys = list(grid)
    out, n = dict(best), 0
    for vals in itertools.product(*(grid[k] for k in keys)):
        spec = dict(zip(keys, vals))
        rt.set_tuning(**launch, blocks_per_sm=0, **spec)
        ms = timer()
        cfg = {**best, **spec, "ms": ms}
        log(json.dumps(cfg))
        n += 1
        if ms < out["ms"]:
            out = cfg
    rt.set_tuning(**launch, blocks_per_sm=0, **{k: out.get(k, 0) for k in keys})
    out["_searched"] = n
    return out


def tune_soups(quick: bool = False, log=print) -> dict:
    """Launch parameters and leaf size of the scene-set trace over the 64-soup workload."""
    import numpy as np
    import torch
    api, wl = _load_pkg()
    tris_n, rays_n = wl.multi_scene_sizes()
    scenes, rays = [], []
    for i, (nt, nr) in enumerate(zip(tris_n, rays_n)):
        sc = wl.soup(1000 + i, nt, sigma=0.5)
        lo, hi = sc.bounds()
        scenes.append((torch.from_numpy(sc.vpos).cuda(), torch.from_numpy(sc.tris.view(np.int32)).cuda()))
        rays.append(torch.from_numpy(wl.shell_rays(2000 + i, lo, hi, nr)).cuda())
    hits = [torch.zeros((r.shape[0], 4), device="cuda") for r in rays]
    batches = [(i, rays[i], hits[i]) for i in range(len(rays))]
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    rt = api.BatchRayTracer(0)
    orders = ["persistent-speculative-while-while"] if quick else ["persistent-while-while",
                                                                  "persistent-speculative-while-while"]
    leaf_sizes = [2] if quick else [2, 3, 4]
    blocks = [64] if quick else [64, 128, 256]
    thresholds = [20] if quick else [8, 12, 16, 20, 24, 28, 32]
    periods = [2] if quick else [1, 2, 4]
    best = None
    t0 = time.time()
    for leaf in leaf_sizes:
        rt.build_scenes_device(scenes, max_tris=leaf, stream=sp)
        for tracer, bt, th, per in itertools.product(orders, blocks, thresholds, periods):
            rt.select(tracer)
            rt.set_tuning(block_threads=bt, refill_threshold=th, refill_period=per, blocks_per_sm=0)
            ms = float("inf")
            for i in range(4):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                rt.trace_multi(batches, stream=sp)
                e1.record(stream)
                e1.synchronize()
                if i:  # the first launch is a warm-up
                    ms = min(ms, e0.elapsed_time(e1))
            rt.check(sp)
            cfg = {"tracer": tracer, "max_tris": leaf, "block_threads": bt, "refill_threshold": th,
                   "refill_period": per, "ms": ms}
            log(json.dumps(cfg))
            if best is None or ms < best["ms"]:
                best = cfg
    searched = len(orders) * len(leaf_sizes) * len(blocks) * len(thresholds) * len(periods)
    if "speculative" in best["tracer"]:
        rt.build_scenes_device(scenes, max_tris=best["max_tris"], stream=sp)
        rt.select(best["tracer"])

        def timer():
            ms = float("inf")
            for i in range(4):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                rt.trace_multi(batches, stream=sp)
                e1.record(stream)
                e1.synchronize()
                if i:
                    ms = min(ms, e0.elapsed_time(e1))
            rt.check(sp)
            return ms

        best = spec_sweep(rt, best, quick, log, timer)
        searched += best.pop("_searched")
    rt.close()
    best["searched"] = searched
    best["seconds"] = round(time.time() - t0, 1)
    return best


def save(best: dict, gpu_name: str, scene: str = "spheres"):
    table = {}
    if os.path.exists(TABLE):
        with open(TABLE) as f:
            table = json.load(f)
    table[f"{gpu_name}|{scene}"] = best
    with open(TABLE, "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--quick", action="store_true")
    ap.add_argument("--paths", type=int, default=4 << 20)
    ap.add_argument("--out", default=None, help="also write the log of every candidate here")
    ap.add_argument("--workload", default="spheres", choices=["spheres", "soups64"])
    a = ap.parse_args()
    import torch
    logf = open(a.out, "w") if a.out else None

    def log(line):
        print(line, flush=True)
        if logf:
            logf.write(line + "\n")

    if a.workload == "soups64":
        best = tune_soups(quick=a.quick, log=log)
    else:
        best = tune(quick=a.quick, n_paths=a.paths, log=log)
    save(best, torch.cuda.get_device_name(0), a.workload)
    log("best " + json.dumps(best))
