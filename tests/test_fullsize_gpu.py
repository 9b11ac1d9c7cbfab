"""Properties at the full sizes of the benchmark configurations, where the oracle would take
too long: the fused persistent path tracer and the plain wavefront agree in every word for all
4,194,304 diffuse paths of the sphere scene (with graphs, exact loop orders), and one launch
over all 64 uneven soups (7,738,242 triangles, 10,745,442 rays) equals 64 single-scene traces
bit for bit, closest and any hit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _needs_cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def test_diffuse_paths_full_size_fused_equals_wavefront(api, wl):
    import torch
    sc, rays_np = wl.spheres_primary(res=1024)
    n_paths = 4 << 20
    rays = torch.from_numpy(rays_np).cuda()
    hits = torch.zeros((rays.shape[0], 4), device="cuda")
    torch.cuda.synchronize()
    side = torch.cuda.Stream()  # graph replay needs a stream of its own
    stream = side.cuda_stream
    out = {}
    for form, tracer, mode in (("wavefront", "while-while", api.PT_WAVEFRONT),
                               ("fused", "persistent-while-while", api.PT_FUSED),
                               ("fused-if-if", "persistent-if-if", api.PT_FUSED)):
        rt = api.BatchRayTracer(0)
        rt.build(sc.vpos, sc.tris)
        rt.select(tracer)
        rt.trace(rays, hits, False, stream)
        res = torch.zeros((n_paths, 4), dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        rt.pathtrace(api.BatchRayTracer.pt_params(mode=mode, use_graph=1), rays, hits, n_paths, res, None, stream)
        rt.check(stream, timeout_ms=120000)
        out[form] = res.cpu().numpy()
        rt.close()
    a = out["wavefront"]
    for form in ("fused", "fused-if-if"):
        assert (a == out[form]).all(), form
    bounces = a[:, 1].astype(np.int64)
    # every path starts at a primary hit (at least one bounce ray), at most 5; the total is the
    # benchmark's bounce-ray count for these seeds
    assert bounces.min() >= 1 and bounces.max() <= 5 and bounces.sum() == 6427617


def test_soups64_one_launch_equals_single_scene_traces(api, wl):
    import torch
    tris_n, rays_n = wl.multi_scene_sizes()
    scenes, rays = [], []
    for i, (nt, nr) in enumerate(zip(tris_n, rays_n)):
        sc = wl.soup(1000 + i, nt, sigma=0.5)
        lo, hi = sc.bounds()
        scenes.append((sc.vpos, sc.tris))
        r = wl.shell_rays(2000 + i, lo, hi, nr)
        rays.append(r)
    assert sum(tris_n) == 7738242 and sum(r.shape[0] for r in rays) == 10745442
    d_rays = [torch.from_numpy(r).cuda() for r in rays]
    stream = torch.cuda.current_stream().cuda_stream
    multi = api.BatchRayTracer(0)
    multi.build_scenes(scenes)
    multi.select("persistent-while-while")
    single = api.BatchRayTracer(0)
    single.select("while-while")
    for any_hit in (False, True):
        if any_hit:  # finite t_max so that occlusion is not trivial
            for r in d_rays:
                r[:, 7] = 2.0
        outs = [torch.zeros((r.shape[0], 4), device="cuda") for r in d_rays]
        multi.trace_multi([(i, d_rays[i], outs[i]) for i in range(len(d_rays))], any_hit=any_hit, stream=stream)
        multi.check(stream, timeout_ms=120000)
        for i, (v, t) in enumerate(scenes):
            single.build(v, t)
            h = torch.zeros_like(outs[i])
            single.trace(d_rays[i], h, any_hit, stream)
            single.check(stream, timeout_ms=120000)
            if any_hit:
                occ_m = outs[i].cpu().numpy().view(np.uint32)[:, 3] == 0xFFFFFFFF
                occ_s = h.cpu().numpy().view(np.uint32)[:, 3] == 0xFFFFFFFF
                assert (occ_m == occ_s).all(), i
            else:
                assert (outs[i].cpu().numpy().view(np.uint32) == h.cpu().numpy().view(np.uint32)).all(), i
    multi.close()
    single.close()
