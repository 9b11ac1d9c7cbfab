#!/usr/bin/env python3
"""Benchmark: Mrays/s closest-hit (coherent + diffuse) on one GB300, tuned persistent vs plain.

Workload (seeded synthetic scene, no external data): 256 UV spheres of 32x16 quads (262,144
triangles), one step =
  * 1024x1024 coherent primary rays, closest hit;
  * 4,194,304 diffuse paths starting at the primary hits, cosine-weighted bounces, at most 5
    bounce rays per path, Russian roulette (continue with p = 0.8) from bounce ray 3 on.
`value` counts every closest-hit ray of the step (primary + bounce rays) per second with the
inputs resident in HBM, using the tuned persistent kernels (persistent primary trace and the
fused traverse+shade+regenerate loop replayed as a CUDA graph). The plain wavefront step (one
thread per ray, one traversal kernel plus one shade kernel per bounce, also as a graph) is timed
beside it. `e2e` runs the same step through the C-ABI from pinned host buffers with the host
copies inside the timed region.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
Multi-GPU (torchrun): every rank runs an independent replica (the path does not shard across
GPUs); value = all ranks' rays / the slowest rank's time.
"""
from __future__ import annotations

import argparse
import gc
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mrays/s closest-hit (coherent+diffuse) on 1 GB300: tuned persistent vs plain wavefront"
WORKLOAD = ("spheres-262144: 1024x1024 coherent primary closest-hit + 4,194,304 diffuse paths "
            "(<=5 bounces, RR p=0.8 from bounce 3)")
RES = 1024
N_PATHS = 4 << 20
LIGHT = (0.0, 15.0, 0.0)
FLT_MAX = 3.4028234663852886e38


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-parity", action="store_true",
                    help="skip the full-size oracle check of the timed configuration")
    ap.add_argument("--profile-case", action="store_true",
                    help="run one tuned and one plain step (no graphs) and exit (for ncu captures)")
    ap.add_argument("--profile-paths", type=int, default=1 << 20, help="paths of the --profile-case step")
    ap.add_argument("--profile-tracer", default=None,
                    help="tracer of the --profile-case step's tuned form instead of the tuning table's")
    ap.add_argument("--workload", default="spheres", choices=["spheres", "soups64", "direct", "adjoint", "gputree"],
                    help="soups64: 64 uneven triangle soups traced in one launch, host vs GPU BVH builds; "
                         "direct: light-source sampling, fused persistent kernel vs wavefront steps; "
                         "adjoint: differentiable hits on the displaced icosphere, one optimisation step "
                         "(tree update, closest hits, adjoint) with a host build, a GPU build or a refit; "
                         "gputree: the tuned spheres step on GPU-built trees (PLOC, radix tree) against the "
                         "host-built tree, with build times")
    return ap.parse_args()


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clock / throttle samples every 100 ms while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.file = None

    def start(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=self.file, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.file.flush()
        rows = []
        with open(self.file.name) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.file.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def measured_hbm_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def tree_options(tuning: dict) -> dict:
    """The reference builder's options of the tuned tree (leaf size, SAH planes, clipping)."""
    return {"max_tris": tuning.get("max_tris", 4), "planes": tuning.get("planes", 16),
            "esc": bool(tuning.get("esc", 1))}


def tree_label(tuning: dict) -> str:
    t = tree_options(tuning)
    return "SAH %d planes, %s, leaf<=%d" % (t["planes"], "ESC" if t["esc"] else "no ESC", t["max_tris"])


def load_tuning(gpu_name: str, scene: str = "spheres") -> dict:
    """The autotuner's entry for this GPU and scene class (the spheres one where there is none)."""
    path = os.path.join(ROOT, "illum-rt_gb300", "tuning.json")
    try:
        with open(path) as f:
            table = json.load(f)
    except Exception:
        return {}
    for key in (f"{gpu_name}|{scene}", f"{gpu_name}|spheres", "default|spheres"):
        if key in table:
            return table[key]
    return {}


def gpu_name_from_smi() -> str:
    """The GPU's name from nvidia-smi (no CUDA context), for the tuning table's key."""
    try:
        out = subprocess.run(["nvidia-smi", "-i", "0", "--query-gpu=name", "--format=csv,noheader"],
                             capture_output=True, text=True, timeout=30)
        name = out.stdout.strip().splitlines()[0].strip() if out.returncode == 0 and out.stdout.strip() else ""
    except Exception:
        name = ""
    return name or "NVIDIA GB300"


def profile_figure(key: str):
    """A figure of the committed ncu summary of the fused kernel (a line `key: N`), or None:
    `dram_bytes_per_launch` (DRAM read + write of one full-size launch) and
    `l2_bytes_per_bounce_ray` (L2 sectors x 32 B per bounce ray)."""
    try:
        with open(os.path.join(ROOT, "profiles", "k_pt_fused_spheres.md")) as f:
            for line in f:
                if line.strip().startswith(key + ":"):
                    return float(line.split(":", 1)[1].strip().replace(",", ""))
    except Exception:
        pass
    return None


def limiter_figures():
    """What bounds the fused kernel instead of HBM, from the committed ncu capture of the
    1,048,576-path case: node-fetch latency and SIMT efficiency (lanes per instruction, issue
    slots busy, L2 throughput)."""
    lanes = profile_figure("lanes_per_instruction")
    issue = profile_figure("issue_active_pct")
    l2 = profile_figure("l2_throughput_pct")
    if lanes is None:
        return None
    return {"kind": "node-fetch latency and SIMT efficiency", "lanes_per_instruction": lanes,
            "issue_active_pct": issue, "l2_throughput_pct": l2,
            "source": "ncu --set full of k_pt_fused, 1,048,576-path case"}


def max_over_ranks(x: float, world: int, device: str = "cuda") -> float:
    """The largest `x` over all ranks (the slowest rank's time); `x` itself for one rank."""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(rays_per_step: int, steps: int, slowest_s: float, world: int) -> float:
    """Whole-job Mrays/s of `world` replicas that each trace `rays_per_step` rays per step."""
    return world * rays_per_step * steps / slowest_s / 1e6


# ---- the GB300 arm --------------------------------------------------------------------------

class Step:
    """Device buffers and the two forms of one benchmark step on one GPU."""

    def __init__(self, api, wl, device: int, tuning: dict):
        import torch
        self.torch = torch
        self.api = api
        sc, rays = wl.spheres_primary(res=RES)
        self.n_primary = rays.shape[0]
        self.rt = api.BatchRayTracer(device)
        tree = tree_options(tuning)
        self.build_info = self.rt.build(sc.vpos, sc.tris, **tree)
        self.rt_plain = api.BatchRayTracer(device)  # the reference's CUDA build defaults, untuned
        self.rt_plain.build(sc.vpos, sc.tris)
        self.rt_plain.select("while-while")
        self.plain_order = "while-while"
        # the plain kernels on the tuned step's tree (its leaf size): the counting pass of the
        # roofline figure and the plain form on the same tree
        self.rt_tt = api.BatchRayTracer(device)
        self.rt_tt.build(sc.vpos, sc.tris, **tree)
        self.rt.select(tuning.get("tracer", "persistent-while-while"))
        kw = {k: v for k, v in tuning.items() if k in api.TUNING_KEYS}
        self.tracer = tuning.get("tracer", "persistent-while-while")
        if kw:
            self.rt.set_tuning(**kw)
        self.dev = torch.device("cuda", device)
        self.h_rays = torch.from_numpy(rays).pin_memory()
        self.rays = self.h_rays.to(self.dev)
        self.hits = torch.zeros((self.n_primary, 4), device=self.dev)
        self.results = torch.zeros((N_PATHS, 4), dtype=torch.int32, device=self.dev)
        self.h_results = torch.zeros((N_PATHS, 4), dtype=torch.int32).pin_memory()
        self.stream = torch.cuda.Stream(self.dev)
        self.sp = self.stream.cuda_stream
        self.p_fused = api.BatchRayTracer.pt_params(mode=api.PT_FUSED, use_graph=1)
        self.p_plain = api.BatchRayTracer.pt_params(mode=api.PT_WAVEFRONT, use_graph=1)
        self.flush_buf = torch.empty(512 << 20, dtype=torch.uint8, device=self.dev)  # > 129 MB of L2

    def flush_l2(self):
        with self.torch.cuda.stream(self.stream):
            self.flush_buf.fill_(1)

    def tuned(self, ev=None):
        self.rt.trace(self.rays, self.hits, False, self.sp)
        if ev is not None:
            ev.record(self.stream)
        self.rt.pathtrace(self.p_fused, self.rays, self.hits, N_PATHS, self.results, None, self.sp)

    def plain(self, ev=None):
        self.rt_plain.trace(self.rays, self.hits, False, self.sp)
        if ev is not None:
            ev.record(self.stream)
        self.rt_plain.pathtrace(self.p_plain, self.rays, self.hits, N_PATHS, self.results, None, self.sp)

    def plain_tuned_tree(self, ev=None):
        self.rt_tt.trace(self.rays, self.hits, False, self.sp)
        if ev is not None:
            ev.record(self.stream)
        self.rt_tt.pathtrace(self.p_plain, self.rays, self.hits, N_PATHS, self.results, None, self.sp)

    def e2e(self):
        with self.torch.cuda.stream(self.stream):
            self.rays.copy_(self.h_rays, non_blocking=True)
            self.rt.trace(self.rays, self.hits, False, self.sp)
            self.rt.pathtrace(self.p_fused, self.rays, self.hits, N_PATHS, self.results, None, self.sp)
            self.h_results.copy_(self.results, non_blocking=True)

    def e2e_pipelined(self, k: int) -> float:
        """K end-to-end steps with the host copies double-buffered across steps: step i copies its
        rays from pinned host memory into a device staging buffer on one stream while step i - 1
        computes, and copies its results back to pinned host memory on another stream while step
        i + 1 computes. The compute stream moves the staged rays into the traced buffer and the
        results out to a staging buffer (device to device), so the captured graph keeps its
        pointers. Returns the wall time of all K steps in ms (first copy in to last copy out)."""
        torch = self.torch
        if not hasattr(self, "stage_in"):
            self.stage_in = [torch.empty_like(self.rays) for _ in range(2)]
            self.stage_out = [torch.empty_like(self.results) for _ in range(2)]
            self.h_out = [torch.empty_like(self.h_results).pin_memory() for _ in range(2)]
            self.s_in, self.s_out = torch.cuda.Stream(self.dev), torch.cuda.Stream(self.dev)
        ev = lambda: torch.cuda.Event()
        in_ready, in_free = [ev(), ev()], [ev(), ev()]
        out_ready, out_free = [ev(), ev()], [ev(), ev()]
        for e in in_free + out_free:
            e.record(self.stream)
        torch.cuda.synchronize()
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record(self.s_in)
        for i in range(k):
            b = i % 2
            with torch.cuda.stream(self.s_in):
                self.s_in.wait_event(in_free[b])
                self.stage_in[b].copy_(self.h_rays, non_blocking=True)
                in_ready[b].record(self.s_in)
            with torch.cuda.stream(self.stream):
                self.stream.wait_event(in_ready[b])
                self.rays.copy_(self.stage_in[b], non_blocking=True)
                in_free[b].record(self.stream)
                self.rt.trace(self.rays, self.hits, False, self.sp)
                self.rt.pathtrace(self.p_fused, self.rays, self.hits, N_PATHS, self.results, None, self.sp)
                self.stream.wait_event(out_free[b])
                self.stage_out[b].copy_(self.results, non_blocking=True)
                out_ready[b].record(self.stream)
            with torch.cuda.stream(self.s_out):
                self.s_out.wait_event(out_ready[b])
                self.h_out[b].copy_(self.stage_out[b], non_blocking=True)
                out_free[b].record(self.s_out)
        self.s_out.wait_stream(self.s_in)
        t1.record(self.s_out)
        t1.synchronize()
        return t0.elapsed_time(t1)

    def rays_per_step(self) -> int:
        self.plain()
        self.rt_plain.check(self.sp)
        bounces = int(self.results[:, 1].sum().item())
        return self.n_primary + bounces

    def algorithmic_bytes(self):
        """(bytes per step of the pathtrace part, bytes of the primary part) from the counting
        kernel on the tuned step's tree: 32 B ray + 16 B hit + 64 B per inner node + 48 B per
        triangle test."""
        torch = self.torch
        cnt = torch.zeros(3, dtype=torch.int64, device=self.dev)
        # the exact reference order, so that the counts are the reference traversal's own
        rt = self.rt_tt
        order = rt.tracer
        rt.select("while-while")
        rt.set_traversal_counters(cnt)
        rt.trace(self.rays, self.hits, False, self.sp)
        rt.check(self.sp)
        prim = [int(x) for x in cnt.cpu()]
        cnt.zero_()
        p = self.api.BatchRayTracer.pt_params(mode=self.api.PT_WAVEFRONT)
        rt.pathtrace(p, self.rays, self.hits, N_PATHS, self.results, None, self.sp)
        rt.check(self.sp)
        bounce = [int(x) for x in cnt.cpu()]
        rt.set_traversal_counters(None)
        rt.select(order)
        to_bytes = lambda c: 48 * c[0] + 64 * c[1] + 48 * c[2]
        return to_bytes(bounce), to_bytes(prim), bounce, prim


def time_steps(step: Step, fn, k: int, flush=True, split=False):
    """Per-step device times (ms) with CUDA events on the step's stream, L2 flushed in between
    (outside the events). With split=True also returns the pathtrace part of each step."""
    torch = step.torch
    totals, parts = [], []
    for _ in range(k):
        if flush:
            step.flush_l2()
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        e0.record(step.stream)
        if split:
            fn(e1)
        else:
            fn()
        e2.record(step.stream)
        e2.synchronize()
        totals.append(e0.elapsed_time(e2))
        if split:
            parts.append(e1.elapsed_time(e2))
    return totals, parts


class CpuStep:
    """One step of the workload on the host cores through the oracle port of the reference CPU
    tracer (OpenMP over rays, rt/cpu/wavefront.cpp:53-70, all host threads): closest hits of the
    1024x1024 primary rays, then the diffuse paths started at those hits. The scene and rays
    come from the oracle's own generators (bit-identical to the library's), and the tree from
    the reference builder with the given options (those of the GPU step's tree), so this loads
    nothing but the oracle."""

    def __init__(self, n_paths: int, tree: dict | None = None, threads: int = 0):
        import __graft_entry__ as ge
        self.orc = ge.load_oracle()
        vpos, tris, self.rays = self.orc.spheres_primary(res=RES)
        self.tree = tree_options(tree or {})
        self.o = self.orc.OracleBVH(vpos, tris, **self.tree)
        self.n_paths = n_paths
        self.threads = threads

    def cores(self) -> int:
        return self.orc.max_threads() if self.threads == 0 else self.threads

    def run(self):
        """(rays traced, seconds) of one step."""
        t0 = time.perf_counter()
        hits, _ = self.o.closest(self.rays, threads=self.threads)
        res, _ = self.o.pathtrace(self.rays, hits, self.n_paths, threads=self.threads)
        dt = time.perf_counter() - t0
        return self.rays.shape[0] + int(res[:, 1].sum()), dt


def cpu_baseline(cs: CpuStep, min_seconds: float = 10.0, min_reps: int = 3):
    """The full step on the host cores, one warm-up step, then repeated until at least
    `min_seconds` of work; the median rate of the repetitions (Mrays/s)."""
    cs.run()
    rates, n_tot, t_tot = [], 0, 0.0
    while t_tot < min_seconds or len(rates) < min_reps:
        n, dt = cs.run()
        rates.append(n / dt / 1e6)
        n_tot += n
        t_tot += dt
    return statistics.median(rates), len(rates), n_tot, t_tot, cs.cores()


NEAR_TIE = 1e-6  # |t1 - t2| <= NEAR_TIE * t: two closest hits equal within float rounding


def classify_hits(got: np.ndarray, want: np.ndarray) -> dict:
    """Hit records float32 [n, 4] (t, beta, gamma, ref bits) against the oracle's: rows whose
    bits differ, and whether each of them is a near-tie (both hit, other triangle, |t1 - t2|
    <= 1e-6 t); a row naming the same triangle with other bits is never a near-tie."""
    g = np.ascontiguousarray(got, np.float32)
    w = np.ascontiguousarray(want, np.float32)
    gu, wu = g.view(np.uint32), w.view(np.uint32)
    rows = np.nonzero((gu != wu).any(axis=1))[0]
    tg, tw = g[rows, 0].astype(np.float64), w[rows, 0].astype(np.float64)
    near = (gu[rows, 3] != wu[rows, 3]) & (tg < 3e38) & (tw < 3e38) & (np.abs(tg - tw) <= NEAR_TIE * np.abs(tw))
    return {"differing": int(rows.size), "all_near_ties": bool(near.all()), "not_near_ties": int((~near).sum())}


def classify_paths(res_g: np.ndarray, bh_g: np.ndarray, res_o: np.ndarray, bh_o: np.ndarray) -> dict:
    """Path results uint32 [n, 4] and bounce-hit records float32 [n, bounces, 4] against the
    oracle's. A path may differ only through a near-tie at its first differing bounce hit
    (from there on it legitimately follows another ray); a path whose results differ while
    all its bounce hits agree, or whose first differing hit is not a near-tie, is a mismatch."""
    ru, ro = np.ascontiguousarray(res_g).view(np.uint32), np.ascontiguousarray(res_o).view(np.uint32)
    bg, bo = np.ascontiguousarray(bh_g, np.float32), np.ascontiguousarray(bh_o, np.float32)
    hit_diff = (bg.view(np.uint32) != bo.view(np.uint32)).any(axis=2)  # [n, bounces]
    paths = np.nonzero((ru != ro).any(axis=1) | hit_diff.any(axis=1))[0]
    d = hit_diff[paths]
    has = d.any(axis=1)
    k = np.argmax(d, axis=1)
    tg = bg[paths, k, 0].astype(np.float64)
    tw = bo[paths, k, 0].astype(np.float64)
    ref_g, ref_o = bg[paths, k, 3].view(np.uint32), bo[paths, k, 3].view(np.uint32)
    near = has & (ref_g != ref_o) & (tg < 3e38) & (tw < 3e38) & (np.abs(tg - tw) <= NEAR_TIE * np.abs(tw))
    return {"differing": int(paths.size), "all_near_ties": bool(near.all()), "not_near_ties": int((~near).sum())}


def oracle_parity(step: Step, cs: CpuStep) -> dict:
    """The timed configuration against the oracle at full size: the tuned step (same tree, tracer,
    launch and graph as the timed loop) once more with its bounce hits recorded, its 1,048,576
    primary hits against the oracle's closest hits, then all 4,194,304 paths against the
    oracle's paths started from the same primary hits. Recording the bounce hits must leave the
    path results of the timed form unchanged."""
    torch = step.torch
    results_timed = step.results.cpu().numpy()
    bh = torch.zeros((N_PATHS, 5, 4), dtype=torch.float32, device=step.dev)
    res = torch.zeros_like(step.results)
    step.rt.trace(step.rays, step.hits, False, step.sp)
    step.rt.pathtrace(step.p_fused, step.rays, step.hits, N_PATHS, res, bh, step.sp)
    step.rt.check(step.sp)
    prim_g = step.hits.cpu().numpy()
    res_g, bh_g = res.cpu().numpy(), bh.cpu().numpy()
    del bh, res
    rays = step.h_rays.numpy()
    same_rays = bool((rays.view(np.uint32) == cs.rays.view(np.uint32)).all())
    prim_o, _ = cs.o.closest(rays)
    prim = classify_hits(prim_g, prim_o)
    res_o, bh_o = cs.o.pathtrace(rays, prim_g, N_PATHS, bounce_hits=True)
    paths = classify_paths(res_g, bh_g, res_o, bh_o)
    timed_equal = bool((results_timed.view(np.uint32) == res_g.view(np.uint32)).all())
    ok = same_rays and timed_equal and prim["all_near_ties"] and paths["all_near_ties"]
    return {"ok": ok, "against": "oracle port of rt/cpu/bvh2.cpp on the same tree (%s)" % tree_label(cs.tree),
            "primary_rays": int(rays.shape[0]), "primary_differing": prim["differing"],
            "primary_exact_or_near_tie": prim["all_near_ties"], "paths": N_PATHS,
            "paths_differing": paths["differing"], "all_near_ties": paths["all_near_ties"],
            "timed_results_equal_recorded": timed_equal, "same_rays": same_rays,
            "near_tie": "other triangle with |t1 - t2| <= 1e-6 t at the first differing hit"}


def rays_in_results(step: Step) -> int:
    return step.n_primary + int(step.results[:, 1].sum().item())


def run_gb300(args):
    import torch
    import __graft_entry__ as ge
    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    ge.load_package()
    from illum_rt_gb300 import api, workloads as wl
    gpu_name = torch.cuda.get_device_name(local)
    tuning = load_tuning(gpu_name)
    step = Step(api, wl, local, tuning)

    # the plain baseline runs in whichever loop order is faster for it (one thread per ray)
    plain_times = {}
    for order in ("while-while", "if-if", "speculative-while-while"):
        step.rt_plain.select(order)
        for _ in range(2):
            step.plain()
        plain_times[order] = statistics.median(time_steps(step, step.plain, 3)[0])
    plain_order = min(plain_times, key=plain_times.get)
    step.plain_order = plain_order
    # for reference only: the same plain wavefront on the 4-wide layout
    step.rt_plain.select("bvh4-speculative-while-while")
    for _ in range(2):
        step.plain()
    plain_bvh4_ms = statistics.median(time_steps(step, step.plain, 3)[0])
    step.rt_plain.select(plain_order)
    # the plain form in its best order on the tuned step's tree
    tt_times = {}
    for order in ("while-while", "if-if", "speculative-while-while"):
        step.rt_tt.select(order)
        for _ in range(2):
            step.plain_tuned_tree()
        tt_times[order] = statistics.median(time_steps(step, step.plain_tuned_tree, 3)[0])
    tt_order = min(tt_times, key=tt_times.get)
    step.rt_tt.select(tt_order)

    # rays per step of each form (identical work: same paths, same bounces)
    step.plain()
    step.rt_plain.check(step.sp)
    rays_plain = rays_in_results(step)
    step.tuned()
    step.rt.check(step.sp)
    rays_tuned = rays_in_results(step)
    pt_bytes, prim_bytes, bounce_cnt, prim_cnt = step.algorithmic_bytes()

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    # warm-up (graphs get captured here)
    for _ in range(max(3, args.warmup)):
        step.tuned()
        step.plain()
        step.plain_tuned_tree()
        step.e2e()
    step.rt.check(step.sp)
    step.rt_plain.check(step.sp)

    # clocks are sampled over all three timed loops (the tuned loop alone is shorter than the
    # sampling period)
    clocks = ClockSampler(local)
    barrier()
    clocks.start()
    # the host must not pause between a step's start event and its launches (the device would
    # idle inside the timed interval): no garbage collection during the timed loops
    gc.collect()
    gc.disable()
    try:
        tuned_ms, pt_ms = time_steps(step, step.tuned, args.steps, split=True)
        barrier()
        plain_ms, plain_pt_ms = time_steps(step, step.plain, args.steps, split=True)
        tt_ms, tt_pt_ms = time_steps(step, step.plain_tuned_tree, args.steps, split=True)
        e2e_ms, _ = time_steps(step, step.e2e, args.steps)
        step.e2e_pipelined(3)  # warm-up of the staging buffers and streams
        e2e_pipe_ms = step.e2e_pipelined(args.steps)
    finally:
        gc.enable()
    barrier()
    clk = clocks.stop()
    step.rt.check(step.sp)
    step.rt_plain.check(step.sp)

    t_tuned = max_over_ranks(sum(tuned_ms) / 1e3, world)
    t_plain = max_over_ranks(sum(plain_ms) / 1e3, world)
    t_e2e = max_over_ranks(sum(e2e_ms) / 1e3, world)
    t_e2e_pipe = max_over_ranks(e2e_pipe_ms / 1e3, world)
    value = job_value(rays_tuned, args.steps, t_tuned, world)
    plain_value = job_value(rays_plain, args.steps, t_plain, world)
    e2e_value = job_value(rays_tuned, args.steps, t_e2e, world)

    # roofline of the dominant kernel (the fused persistent loop): algorithmic bytes of all its
    # bounce rays per launch / the pathtrace part of each timed step
    peak, peak_kind = measured_hbm_peak()
    pt_s = statistics.mean(pt_ms) / 1e3
    achieved = pt_bytes / pt_s / 1e9
    traffic = profile_figure("dram_bytes_per_launch")
    l2_per_ray = profile_figure("l2_bytes_per_bounce_ray")
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": int(traffic) if traffic is not None else None,
                "kernel": "k_pt_fused", "peak_source": peak_kind,
                "bytes_per_launch": pt_bytes, "bounce_rays": bounce_cnt[0],
                "inner_nodes_per_ray": round(bounce_cnt[1] / max(1, bounce_cnt[0]), 2),
                "tri_tests_per_ray": round(bounce_cnt[2] / max(1, bounce_cnt[0]), 2),
                "l2_gbs": round(l2_per_ray * bounce_cnt[0] / pt_s / 1e9, 1) if l2_per_ray else None,
                "l2_note": "L2 bytes per bounce ray from the ncu capture of the 1,048,576-path case x this "
                           "launch's bounce rays / its measured time",
                "note": "B_ray = 32 + 16 + 64 n_node + 48 n_tri, counted in the exact while-while order on the "
                        "tuned step's tree; the BVH (%.0f MB) stays L2-resident, so these bytes are mostly served "
                        "from L2" % (step.build_info["device_bytes"] / 1e6),
                "limiter": limiter_figures()}
    line = {
        "metric": METRIC, "value": round(value, 1), "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(statistics.mean(tuned_ms), 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD, "triangles": 262144, "primary_rays": step.n_primary, "paths": N_PATHS,
                   "rays_per_step": rays_tuned, "bvh": tree_label(tuning),
                   "l2": "flushed between timed steps (512 MB write); the pipelined e2e loop adds no flush, each "
                         "of its steps moves about 256 MB of copies and results through L2",
                   "parallelism": f"replicas x{world}",
                   "tuning": tuning or "defaults"},
        "step_ms_spread": {"tuned": [round(min(tuned_ms), 4), round(statistics.median(tuned_ms), 4),
                                     round(max(tuned_ms), 4)],
                           "plain": [round(min(plain_ms), 4), round(statistics.median(plain_ms), 4),
                                     round(max(plain_ms), 4)],
                           "plain_same_tree": [round(min(tt_ms), 4), round(statistics.median(tt_ms), 4),
                                               round(max(tt_ms), 4)],
                           "form": "min, median, max of the timed steps"},
        "plain_wavefront": {"value": round(plain_value, 1), "ms_per_step": round(statistics.mean(plain_ms), 4),
                            "rays_per_step": rays_plain, "loop_order": plain_order,
                            "order_ms": {k: round(v, 4) for k, v in plain_times.items()},
                            "bvh4_speculative_ms": round(plain_bvh4_ms, 4),
                            "tuned_tree": {"bvh": tree_label(tuning),
                                           "loop_order": tt_order, "ms_per_step": round(statistics.mean(tt_ms), 4),
                                           "order_ms": {k: round(v, 4) for k, v in tt_times.items()}}},
        "speedup_vs_plain": round(value / plain_value, 3),
        "speedup_vs_plain_same_tree": round(statistics.mean(tt_ms) / statistics.mean(tuned_ms), 3),
        "speedup_vs_plain_while_while": round(plain_times["while-while"] / statistics.mean(tuned_ms), 3),
        "diffuse_only": {
            "rays_per_step": rays_tuned - step.n_primary,
            "tuned_ms": round(statistics.mean(pt_ms), 4),
            "plain_ms": round(statistics.mean(plain_pt_ms), 4),
            "plain_same_tree_ms": round(statistics.mean(tt_pt_ms), 4),
            "Mrays_s": round((rays_tuned - step.n_primary) / statistics.mean(pt_ms) / 1e3, 1),
            "speedup_vs_plain": round(statistics.mean(plain_pt_ms) / statistics.mean(pt_ms), 3),
            "speedup_vs_plain_same_tree": round(statistics.mean(tt_pt_ms) / statistics.mean(pt_ms), 3),
            "spread_ms": {"tuned": [round(min(pt_ms), 4), round(max(pt_ms), 4)],
                          "plain_same_tree": [round(min(tt_pt_ms), 4), round(max(tt_pt_ms), 4)]},
            "form": "the diffuse bounce part of each timed step alone (after the primary trace), L2 flushed "
                    "before each step"},
        "e2e": {"value": round(job_value(rays_tuned, args.steps, t_e2e_pipe, world), 1), "unit": "Mrays/s",
                "ms_per_step": round(e2e_pipe_ms / args.steps, 4), "h2d_bytes_per_step": int(step.n_primary * 32),
                "d2h_bytes_per_step": int(N_PATHS * 16),
                "form": "host copies double-buffered across steps on two copy streams",
                "serial": {"value": round(e2e_value, 1), "ms_per_step": round(statistics.mean(e2e_ms), 4),
                           "form": "copy in, step, copy out on one stream"}},
        "gpu_launches": 6 * args.steps,
        "roofline": roofline,
        "clocks": clk,
        "build_ms": round(step.build_info["build_ms"], 1),
    }
    cs = None
    if rank == 0 and (not args.no_parity or (world == 1 and not args.no_cpu_baseline)):
        cs = CpuStep(N_PATHS, tuning)
    if cs is not None and not args.no_parity:
        line["parity"] = oracle_parity(step, cs)
    if cs is not None and world == 1 and not args.no_cpu_baseline:
        v, reps, n, dt, cores = cpu_baseline(cs)
        line["cpu_baseline"] = {"value": round(v, 2), "unit": "Mrays/s", "cores": cores, "kind": "port",
                                "sample": f"the full step (1024x1024 primary rays + 4,194,304 diffuse paths, "
                                          f"{tree_label(tuning)}) x {reps} after 1 warm-up: {n} rays in {dt:.1f} s, "
                                          f"median rate"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


# ---- the reference arm: the reference's CPU tracer (oracle port) on the host cores ------------

def run_reference(args):
    """The reference's CPU tracer (the oracle port of rt/cpu/bvh2.cpp and wavefront.cpp) on the
    host cores, rank 0 only: every step is the full workload (closest hits of the primary rays
    and the diffuse paths from them)."""
    rank, world, _ = dist_info()
    if rank != 0:
        return
    tuning = load_tuning(gpu_name_from_smi())
    cs = CpuStep(N_PATHS, tuning)
    rays = cs.rays
    for _ in range(args.warmup):
        cs.run()
    n_tot, t_tot = 0, 0.0
    for _ in range(args.steps):
        n, dt = cs.run()
        n_tot += n
        t_tot += dt
    value = n_tot / t_tot / 1e6
    cores = cs.cores()
    line = {"metric": METRIC, "value": round(value, 2), "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(1e3 * t_tot / args.steps, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)", "impl": "reference",
            "config": {"workload": WORKLOAD, "triangles": 262144, "primary_rays": rays.shape[0], "paths": N_PATHS,
                       "rays_per_step": n_tot // max(1, args.steps), "bvh": tree_label(tuning)},
            "cpu_baseline": {"value": round(value, 2), "unit": "Mrays/s", "cores": cores, "kind": "port",
                             "sample": f"the full step x {args.steps} after {args.warmup} warm-up, OpenMP over rays"},
            "ref_source": "oracle port of rt/cpu/bvh2.cpp and rt/cpu/wavefront.cpp:53-70 (its trees and hits pinned "
                          "to the reference compiled from its sources, tests/golden), scene and rays from the "
                          "oracle's own generators; the reference's CPU build needs its sources, absent on this host",
            "e2e": {"value": round(value, 2), "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_soups64(args):
    """64 triangle soups of log-uniform size in [1,024, 1,048,576] triangles with log-uniform ray
    batches in [4,096, 1,048,576] (7,738,242 triangles, 10,745,442 rays), all batches in one
    persistent launch. Reports the wall time of the host build (the reference builder, scenes in
    parallel) and of the GPU builds (radix tree, and PLOC clustering), and the trace rate on
    each tree."""
    import torch
    import __graft_entry__ as ge
    ge.load_package()
    from illum_rt_gb300 import api, workloads as wl
    tris_n, rays_n = wl.multi_scene_sizes()
    scenes, rays = [], []
    for i, (nt, nr) in enumerate(zip(tris_n, rays_n)):
        sc = wl.soup(1000 + i, nt, sigma=0.5)
        lo, hi = sc.bounds()
        scenes.append((sc.vpos, sc.tris))
        rays.append(wl.shell_rays(2000 + i, lo, hi, nr))
    d_scenes = [(torch.from_numpy(v).cuda(), torch.from_numpy(t.view(np.int32)).cuda()) for v, t in scenes]
    d_rays = [torch.from_numpy(r).cuda() for r in rays]
    hits = [torch.zeros((r.shape[0], 4), device="cuda") for r in rays]
    n_rays = sum(r.shape[0] for r in rays)
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    tuning = load_tuning(torch.cuda.get_device_name(0), "soups64")
    out = {"metric": "Mrays/s closest-hit, 64 uneven soups in one launch", "unit": "Mrays/s", "n_gpus": 1,
           "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "dtype": "f32",
           "data": "synthetic (seeded)",
           "config": {"workload": "soups64", "scenes": 64, "triangles": int(sum(tris_n)), "rays": int(n_rays),
                      "tuning": tuning or "defaults",
                      "l2": "inputs (344 MB of rays) larger than L2"}}

    def timed_trace(rt):
        batches = [(i, d_rays[i], hits[i]) for i in range(len(rays))]
        for _ in range(max(3, args.warmup)):
            rt.trace_multi(batches, stream=sp)
        rt.check(sp)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            rt.trace_multi(batches, stream=sp)
        e1.record(stream)
        e1.synchronize()
        rt.check(sp)
        return e0.elapsed_time(e1) / args.steps

    for kind in ("host", "gpu", "gpu_ploc", "gpu_lbvh"):
        rt = api.BatchRayTracer(0)
        if kind == "gpu_ploc":
            rt.set_device_builder("ploc")
        elif kind == "gpu_lbvh":
            rt.set_device_builder("lbvh")
        rt.select(tuning.get("tracer", "persistent-speculative-while-while"))
        kw = {k: v for k, v in tuning.items() if k in api.TUNING_KEYS}
        if kw:
            rt.set_tuning(**kw)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        if kind == "host":
            rt.build_scenes(scenes, max_tris=tuning.get("max_tris", 4))
        else:  # the default device builder (SAH splits), PLOC clustering or the radix tree
            rt.build_scenes_device(d_scenes, max_tris=tuning.get("max_tris", 4), stream=sp)
        build_s = time.perf_counter() - t0
        ms = timed_trace(rt)
        out[kind + "_tree"] = {"build_s": round(build_s, 4), "trace_ms": round(ms, 4),
                               "Mrays_s": round(n_rays / ms / 1e3, 1),
                               "end_to_end_s": round(build_s + ms / 1e3, 4)}
        rt.close()
    out["value"] = out["gpu_tree"]["Mrays_s"]
    out["build_speedup_gpu_vs_host"] = round(out["host_tree"]["build_s"] / out["gpu_tree"]["build_s"], 1)
    out["host_threads"] = os.cpu_count()
    print(json.dumps(out), flush=True)


def run_direct(args, samples: int = 8):
    """Direct lighting on the 256 spheres with a floor and two area lights, 1024x1024 camera
    rays, `samples` light samples per pixel: the fused persistent kernel against the wavefront
    steps (camera trace, then per sample: light sampling, shadow trace, integration) in the
    fastest exact loop order for each. Value: light samples per second of the fused form."""
    import torch
    import __graft_entry__ as ge
    ge.load_package()
    from illum_rt_gb300 import api, workloads as wl
    sc, mats, rays_np = wl.lit_spheres(count=256, res=RES)
    n = rays_np.shape[0]
    rays = torch.from_numpy(rays_np).cuda()
    fb = torch.zeros((n, 4), device="cuda")
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    rt = api.BatchRayTracer(0)
    # the reference default tree: on this scene (a floor of two large triangles under the
    # spheres) the builder's split clipping pays; without it the fused frame took 2.78 ms
    # instead of 2.38 ms
    rt.build(sc.vpos, sc.tris)
    rt.set_material_table(mats)
    flush_buf = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")  # > 129 MB of L2

    def timed(mode, tracer, sampling="light"):
        rt.select(tracer)
        for _ in range(max(3, args.warmup)):
            rt.direct(rays, fb, samples, mode=mode, seed=3, stream=sp, sampling=sampling)
        rt.check(sp)
        times = []
        for _ in range(args.steps):
            with torch.cuda.stream(stream):
                flush_buf.fill_(1)  # L2 flushed between timed frames, outside the events
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            rt.direct(rays, fb, samples, mode=mode, seed=3, stream=sp, sampling=sampling)
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
        rt.check(sp)
        return statistics.median(times)

    res = {}
    for tracer in ("while-while", "if-if", "speculative-while-while", "bvh4-speculative-while-while"):
        res["fused/" + tracer] = timed(api.DL_FUSED, tracer)
    for tracer in ("while-while", "if-if", "speculative-while-while", "persistent-speculative-while-while"):
        res["wavefront/" + tracer] = timed(api.DL_WAVEFRONT, tracer)
    best_f = min((v, k) for k, v in res.items() if k.startswith("fused"))
    best_w = min((v, k) for k, v in res.items() if k.startswith("wavefront"))
    # the direction strategies of direct-wf (closest-hit rays instead of shadow rays), in the
    # loop orders that are fastest for light sampling
    directions = {}
    for smp in ("uniform", "cosine"):
        f_ms = timed(api.DL_FUSED, best_f[1].split("/", 1)[1], smp)
        w_ms = timed(api.DL_WAVEFRONT, best_w[1].split("/", 1)[1], smp)
        directions[smp] = {"fused_ms": round(f_ms, 4), "wavefront_ms": round(w_ms, 4),
                           "speedup_fused_vs_wavefront": round(w_ms / f_ms, 3)}
    line = {"metric": "Msamples/s direct lighting (light-source sampling), fused vs wavefront", "unit": "Msamples/s",
            "value": round(n * samples / best_f[0] / 1e3, 1), "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": "lit_spheres-262150: 256 spheres, floor, 2 area lights, 1024x1024 camera rays",
                       "samples_per_pixel": samples,
                       "l2": "flushed between timed frames (512 MB write)"},
            "fused_ms": round(best_f[0], 4), "fused_form": best_f[1], "wavefront_ms": round(best_w[0], 4),
            "wavefront_form": best_w[1], "speedup_fused_vs_wavefront": round(best_w[0] / best_f[0], 3),
            "all_ms": {k: round(v, 4) for k, v in res.items()}, "direction_sampling": directions}
    print(json.dumps(line), flush=True)
    rt.close()


def run_adjoint(args):
    """Differentiable closest hits on the displaced icosphere (81,920 triangles, 512x512 camera
    rays): one step of a gradient descent on the vertices = moving the vertices, updating the
    tree, the closest hits and the adjoint (dL/dvertices, dL/drays) of a loss on (t, beta,
    gamma). The tree update is a host build (the reference's way), a GPU build or a refit; the
    vertices move every step, so every form does its update every step. Value: rays per second
    of the refit form."""
    import torch
    import __graft_entry__ as ge
    ge.load_package()
    from illum_rt_gb300 import api, workloads as wl
    sc, rays_np = wl.icosphere_primary(res=512)
    n = rays_np.shape[0]
    rays = torch.from_numpy(rays_np).cuda()
    tris = torch.from_numpy(sc.tris.view(np.int32)).cuda()
    v0 = torch.from_numpy(sc.vpos).cuda()
    step_dir = torch.from_numpy(np.random.default_rng(6).normal(size=sc.vpos.shape).astype(np.float32)).cuda()
    step_dir[:, 3] = 0.0
    hits = torch.zeros((n, 4), device="cuda")
    g3 = torch.from_numpy(np.random.default_rng(7).normal(size=(n, 3)).astype(np.float32)).cuda()
    gv = torch.zeros((sc.vpos.shape[0], 3), device="cuda")
    gr = torch.zeros((n, 8), device="cuda")
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    tuning = load_tuning(torch.cuda.get_device_name(0))
    tracer = tuning.get("tracer", "persistent-speculative-while-while")

    def run(form):
        rt = api.BatchRayTracer(0)
        rt.select(tracer)
        rt.build_device(v0, tris, stream=sp)
        vhost = sc.vpos.copy()

        def one(i):
            v = v0 + (1e-4 * (i % 7)) * step_dir
            if form == "host":
                vhost[:, :3] = v[:, :3].cpu().numpy()
                rt.build(vhost, sc.tris)
            elif form == "gpu":
                rt.build_device(v, tris, stream=sp)
            else:
                rt.refit(v, stream=sp)
            rt.trace(rays, hits, False, sp)
            gv.zero_()
            rt.adjoint(rays, hits, g3, gv, gr, vpos=v, stream=sp)

        with torch.cuda.stream(stream):
            for i in range(max(3, args.warmup)):
                one(i)
            rt.check(sp)
            torch.cuda.synchronize()
            steps = args.steps if form != "host" else max(3, min(args.steps, 10))
            t0 = time.perf_counter()
            for i in range(steps):
                one(i)
            rt.check(sp)
            torch.cuda.synchronize()
            ms = (time.perf_counter() - t0) * 1e3 / steps
        rt.close()
        return ms

    res = {form: run(form) for form in ("refit", "gpu", "host")}
    line = {"metric": "Mrays/s differentiable closest hits (tree update + trace + adjoint per step)",
            "unit": "Mrays/s", "value": round(n / res["refit"] / 1e3, 1), "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": "icosphere-81920 (6 subdivisions, radial displacement 0.05), 512x512 rays",
                       "tracer": tracer, "timing": "host wall clock per step, synchronised"},
            "ms_per_step": {k: round(v, 4) for k, v in res.items()},
            "speedup_refit_vs_host_build": round(res["host"] / res["refit"], 1),
            "speedup_refit_vs_gpu_build": round(res["gpu"] / res["refit"], 2)}
    print(json.dumps(line), flush=True)


def run_gputree(args):
    """The tuned spheres step (persistent primary trace + fused loop, L2 flushed before each step) on
    the host-built tuned tree and on trees built on the GPU from device arrays by the SAH builder
    (the tuned tree's plane count), by PLOC and by the radix tree, leaves of at most 1-4; build
    wall times, also for a 1,048,576-triangle soup."""
    import torch
    import __graft_entry__ as ge
    ge.load_package()
    from illum_rt_gb300 import api, workloads as wl
    step = Step(api, wl, 0, load_tuning(torch.cuda.get_device_name(0)))
    sc, _ = wl.spheres_primary(res=RES)
    v = torch.from_numpy(sc.vpos).cuda()
    t = torch.from_numpy(sc.tris.view(np.int32)).cuda()
    out = {"metric": "ms per tuned spheres step on GPU-built trees", "unit": "ms", "higher_is_better": False,
           "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "data": "synthetic (seeded)",
           "config": {"workload": WORKLOAD, "l2": "flushed between timed steps"}, "trees": {}}

    def timed():
        for _ in range(max(3, args.warmup)):
            step.tuned()
        step.rt.check(step.sp)
        gc.disable()
        try:
            tot, part = time_steps(step, step.tuned, args.steps, split=True)
        finally:
            gc.enable()
        return {"step_ms": round(statistics.mean(tot), 4), "fused_ms": round(statistics.mean(part), 4)}

    tuning = load_tuning(torch.cuda.get_device_name(0))
    out["trees"]["host"] = dict(timed(), bvh=tree_label(tuning))
    planes = min(256, int(tree_options(tuning)["planes"]))
    for builder in ("sah", "ploc", "lbvh"):
        for leaf in (1, 2, 3, 4):
            step.rt.set_device_builder(builder, planes=planes)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            info = step.rt.build_device(v, t, max_tris=leaf, stream=step.sp)
            build_ms = (time.perf_counter() - t0) * 1e3
            out["trees"][f"{builder}_leaf{leaf}"] = dict(timed(), build_ms=round(build_ms, 2), depth=info["depth"],
                                                         inner_nodes=info["inner_nodes"])
    s = wl.soup(1000, 1 << 20)
    sv, st = torch.from_numpy(s.vpos).cuda(), torch.from_numpy(s.tris.view(np.int32)).cuda()
    rt = api.BatchRayTracer(0)
    for builder in ("sah", "ploc", "lbvh"):
        rt.set_device_builder(builder, planes=planes)
        rt.build_device(sv, st, max_tris=2)  # warm-up of the allocations
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rt.build_device(sv, st, max_tris=2)
        out[f"soup_1048576_{builder}_build_ms"] = round((time.perf_counter() - t0) * 1e3, 2)
    rt.close()
    print(json.dumps(out), flush=True)


def run_profile_case(paths: int, tracer: str | None = None):
    """One tuned step, then one plain step on the same tree in the speculative order (no graphs;
    1,048,576 paths unless asked otherwise): a case whose launches ncu can capture one by one.
    `tracer` replaces the tuned form's tracer (the tuning table's launch parameters stay)."""
    import torch
    import __graft_entry__ as ge
    global N_PATHS
    N_PATHS = paths
    ge.load_package()
    from illum_rt_gb300 import api, workloads as wl
    tuning = load_tuning(torch.cuda.get_device_name(0))
    if tracer:
        tuning = dict(tuning, tracer=tracer)
    step = Step(api, wl, 0, tuning)
    step.rt_tt.select("speculative-while-while")  # the plain form's fastest order on GB300
    step.p_fused.use_graph = 0
    step.p_plain.use_graph = 0
    step.tuned()
    step.plain_tuned_tree()
    step.rt.check(step.sp)
    step.rt_tt.check(step.sp)
    print(json.dumps({"profile_case": "ok", "paths": N_PATHS, "rays": rays_in_results(step)}))


def run_profile_case_other(workload: str):
    """One launch of the dominant kernel of the direct or soups64 workload at full size, for ncu:
    direct: the fused direct-lighting kernel (speculative order, 8 light samples, 1024x1024);
    soups64: the scene-set trace of all 64 soups (GPU-built trees)."""
    import torch
    import __graft_entry__ as ge
    ge.load_package()
    from illum_rt_gb300 import api, workloads as wl
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    tuning = load_tuning(torch.cuda.get_device_name(0), workload)
    rt = api.BatchRayTracer(0)
    if workload == "direct":
        sc, mats, rays_np = wl.lit_spheres(count=256, res=RES)
        rays = torch.from_numpy(rays_np).cuda()
        fb = torch.zeros((rays.shape[0], 4), device="cuda")
        rt.build(sc.vpos, sc.tris)
        rt.set_material_table(mats)
        rt.select("speculative-while-while")
        rt.direct(rays, fb, 8, mode=api.DL_FUSED, seed=3, stream=sp)
        n = rays.shape[0] * 8
    else:
        tris_n, rays_n = wl.multi_scene_sizes()
        scenes, rays = [], []
        for i, (nt, nr) in enumerate(zip(tris_n, rays_n)):
            sc = wl.soup(1000 + i, nt, sigma=0.5)
            lo, hi = sc.bounds()
            scenes.append((torch.from_numpy(sc.vpos).cuda(), torch.from_numpy(sc.tris.view(np.int32)).cuda()))
            rays.append(torch.from_numpy(wl.shell_rays(2000 + i, lo, hi, nr)).cuda())
        hits = [torch.zeros((r.shape[0], 4), device="cuda") for r in rays]
        rt.select(tuning.get("tracer", "persistent-speculative-while-while"))
        kw = {k: v for k, v in tuning.items() if k in api.TUNING_KEYS}
        if kw:
            rt.set_tuning(**kw)
        rt.build_scenes_device(scenes, max_tris=tuning.get("max_tris", 4), stream=sp)
        rt.trace_multi([(i, rays[i], hits[i]) for i in range(len(rays))], stream=sp)
        n = sum(r.shape[0] for r in rays)
    rt.check(sp)
    rt.close()
    print(json.dumps({"profile_case": "ok", "workload": workload, "units": int(n)}))


def main():
    args = parse_args()
    if args.profile_case and args.workload in ("direct", "soups64"):
        run_profile_case_other(args.workload)
    elif args.profile_case:
        run_profile_case(args.profile_paths, args.profile_tracer)
    elif args.impl == "reference":
        run_reference(args)
    elif args.workload == "soups64":
        run_soups64(args)
    elif args.workload == "direct":
        run_direct(args)
    elif args.workload == "adjoint":
        run_adjoint(args)
    elif args.workload == "gputree":
        run_gputree(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
