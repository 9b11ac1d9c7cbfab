"""Per-call device timers (grt_set_timing / grt_timing_stats, the counterpart of the reference's
wavefront step timers): off by default, one count per call and kind while on, device times
that add up, a reset, and no recording while a stream is being captured into a graph."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _needs_cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def test_call_timers(api, wl):
    import torch
    sc, rays_np = wl.spheres_primary(res=512)
    rays = torch.from_numpy(rays_np).cuda()
    hits = torch.zeros((rays.shape[0], 4), device="cuda")
    side = torch.cuda.Stream()
    sp = side.cuda_stream
    rt = api.BatchRayTracer(0)
    rt.build(sc.vpos, sc.tris)
    rt.select("persistent-speculative-while-while")
    rt.trace(rays, hits, False, sp)
    assert all(c == 0 for c, _ in rt.timing_stats().values())  # off by default
    rt.set_timing(True)
    for _ in range(5):
        rt.trace(rays, hits, False, sp)
    res = torch.zeros((1 << 18, 4), dtype=torch.int32, device="cuda")
    for _ in range(2):
        rt.pathtrace(api.BatchRayTracer.pt_params(mode=api.PT_FUSED, use_graph=1), rays, hits, 1 << 18, res, None, sp)
    rt.check(sp)
    st = rt.timing_stats()
    assert st["trace"][0] == 5 and st["pathtrace"][0] == 2 and st["direct"][0] == 0
    assert 0 < st["trace"][1] < 5000 and 0 < st["pathtrace"][1] < 5000
    # a kernel's own events agree with the timer: the timed calls cover at least the kernel time
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(side)
    rt.trace(rays, hits, False, sp)
    e1.record(side)
    e1.synchronize()
    st2 = rt.timing_stats(reset=True)
    assert st2["trace"][0] == 6
    one = st2["trace"][1] - st["trace"][1]
    assert 0 < one <= e0.elapsed_time(e1) * 1.05 + 0.05
    assert all(c == 0 for c, _ in rt.timing_stats().values())  # after the reset
    # calls issued while the stream is being captured into a graph are not timed
    rt.select("while-while")
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        rt.trace(rays, hits, False, torch.cuda.current_stream().cuda_stream)
    g.replay()
    torch.cuda.synchronize()
    assert rt.timing_stats()["trace"][0] == 0
    rt.set_timing(False)
    rt.trace(rays, hits, False, sp)
    rt.check(sp)
    assert rt.timing_stats()["trace"][0] == 0
    rt.close()
