"""Stopping work early (grt_abort, grt_check with a time limit), without faulting or hanging
the GPU: the request is two words written by the copy engine, the persistent kernels read them
at entry and through their work counter, and the context is usable again after the check that
reports the stop. The reference cannot stop a launch; its error path resets the device
(rt/cuda/cuda-helpers.cpp:5-12)."""
import threading
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ABORTED, TIMEOUT = 11, 4
PERSISTENT = ("persistent-while-while", "persistent-speculative-while-while")


@pytest.fixture(autouse=True)
def _needs_cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


@pytest.fixture(scope="module")
def spheres(wl):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    sc, rays_np = wl.spheres_primary(res=1024)
    return sc, torch.from_numpy(rays_np).cuda()


def _status(api, fn):
    with pytest.raises(api.GRTError) as e:
        fn()
    return e.value.status


@pytest.mark.parametrize("tracer", PERSISTENT)
def test_abort_before_launch_skips_work_then_context_recovers(api, spheres, tracer):
    import torch
    sc, rays = spheres
    stream = torch.cuda.current_stream().cuda_stream
    rt = api.BatchRayTracer(0)
    rt.build(sc.vpos, sc.tris)
    rt.select(tracer)
    want = torch.zeros((rays.shape[0], 4), device="cuda")
    rt.trace(rays, want, False, stream)
    rt.check(stream, timeout_ms=60000)
    rt.abort()
    hits = torch.zeros_like(want)
    rt.trace(rays, hits, False, stream)
    assert _status(api, lambda: rt.check(stream, timeout_ms=60000)) == ABORTED
    assert (hits == 0).all()  # the launch took no rays
    rt.check(stream, timeout_ms=60000)  # the request was cleared
    rt.trace(rays, hits, False, stream)
    rt.check(stream, timeout_ms=60000)
    assert torch.equal(hits.view(torch.int32), want.view(torch.int32))
    rt.close()


def test_abort_before_launch_skips_scene_set(api, wl):
    import torch
    scenes, rays = [], []
    for i in range(4):
        sc = wl.soup(500 + i, 4096 << i, sigma=0.5)
        lo, hi = sc.bounds()
        scenes.append((sc.vpos, sc.tris))
        rays.append(torch.from_numpy(wl.shell_rays(600 + i, lo, hi, 8192)).cuda())
    stream = torch.cuda.current_stream().cuda_stream
    rt = api.BatchRayTracer(0)
    rt.build_scenes(scenes)
    rt.select("persistent-while-while")
    want = [torch.zeros((r.shape[0], 4), device="cuda") for r in rays]
    rt.trace_multi([(i, rays[i], want[i]) for i in range(4)], any_hit=False, stream=stream)
    rt.check(stream, timeout_ms=60000)
    rt.abort()
    got = [torch.zeros_like(w) for w in want]
    rt.trace_multi([(i, rays[i], got[i]) for i in range(4)], any_hit=False, stream=stream)
    assert _status(api, lambda: rt.check(stream, timeout_ms=60000)) == ABORTED
    assert all((g == 0).all() for g in got)
    rt.trace_multi([(i, rays[i], got[i]) for i in range(4)], any_hit=False, stream=stream)
    rt.check(stream, timeout_ms=60000)
    for g, w in zip(got, want):
        assert torch.equal(g.view(torch.int32), w.view(torch.int32))
    rt.close()


def _fused_paths(api, spheres, n_paths):
    """A context with the fused path tracer ready, the primary hits, and a complete run."""
    import torch
    sc, rays = spheres
    side = torch.cuda.Stream()
    stream = side.cuda_stream
    rt = api.BatchRayTracer(0)
    rt.build(sc.vpos, sc.tris)
    rt.select("persistent-while-while")
    hits = torch.zeros((rays.shape[0], 4), device="cuda")
    rt.trace(rays, hits, False, stream)
    params = api.BatchRayTracer.pt_params(mode=api.PT_FUSED, use_graph=0)
    full = torch.zeros((n_paths, 4), dtype=torch.int32, device="cuda")
    rt.pathtrace(params, rays, hits, n_paths, full, None, stream)
    rt.check(stream, timeout_ms=120000)
    return rt, stream, params, hits, full


def _check_partial(part, full):
    """Paths are either finished, equal to the complete run, or untouched (all zero)."""
    p, f = part.cpu().numpy(), full.cpu().numpy()
    done = p[:, 1] > 0  # every path of this scene starts at a primary hit: one bounce ray at least
    assert (p[done] == f[done]).all()
    assert (p[~done] == 0).all()
    return int(done.sum())


def test_check_time_limit_stops_fused_path_tracer(api, spheres):
    import torch
    sc, rays = spheres
    n_paths = 16 << 20
    rt, stream, params, hits, full = _fused_paths(api, spheres, n_paths)
    part = torch.zeros_like(full)
    rt.pathtrace(params, rays, hits, n_paths, part, None, stream)
    t0 = time.perf_counter()
    assert _status(api, lambda: rt.check(stream, timeout_ms=1)) == TIMEOUT
    waited = time.perf_counter() - t0
    done = _check_partial(part, full)
    assert done < n_paths, "the time limit stopped nothing"
    assert waited < 2.5, waited
    # the request is cleared and the context runs the same work to the end again
    rt.pathtrace(params, rays, hits, n_paths, part, None, stream)
    rt.check(stream, timeout_ms=120000)
    assert torch.equal(part, full)
    rt.close()


def test_abort_from_another_thread_stops_a_wait(api, spheres):
    import torch
    sc, rays = spheres
    n_paths = 32 << 20
    rt, stream, params, hits, full = _fused_paths(api, spheres, n_paths)
    part = torch.zeros_like(full)
    rt.pathtrace(params, rays, hits, n_paths, part, None, stream)
    watchdog = threading.Timer(0.003, rt.abort)
    watchdog.start()
    status = _status(api, lambda: rt.check(stream, timeout_ms=60000))
    watchdog.join()
    assert status == ABORTED
    done = _check_partial(part, full)
    assert done < n_paths
    rt.pathtrace(params, rays, hits, n_paths, part, None, stream)
    rt.check(stream, timeout_ms=120000)
    assert torch.equal(part, full)
    rt.close()


def test_plain_tracer_runs_to_the_end_under_a_request(api, spheres):
    """One-thread-per-ray launches are bounded by their ray count and are not stopped; the
    check still reports the request and clears it."""
    import torch
    sc, rays = spheres
    stream = torch.cuda.current_stream().cuda_stream
    rt = api.BatchRayTracer(0)
    rt.build(sc.vpos, sc.tris)
    rt.select("while-while")
    want = torch.zeros((rays.shape[0], 4), device="cuda")
    rt.trace(rays, want, False, stream)
    rt.check(stream, timeout_ms=60000)
    rt.abort()
    hits = torch.zeros_like(want)
    rt.trace(rays, hits, False, stream)
    assert _status(api, lambda: rt.check(stream, timeout_ms=60000)) == ABORTED
    assert torch.equal(hits.view(torch.int32), want.view(torch.int32))
    rt.check(stream, timeout_ms=60000)
    rt.close()
