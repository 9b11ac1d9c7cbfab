"""GPU BVH construction (grt_build_device, grt_build_scenes_device): trees built on the GPU
from device arrays, with each tree builder (top-down SAH, PLOC clustering and the Morton radix
tree), traced by every tracer, against the oracle on the reference's tree.
Closest hits may differ from the reference only as near-ties (another tree visits triangles in
another order); any-hit answers are equal. Also: degenerate inputs, errors, and the statistics
of the trees."""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, assert_hits_match

pytestmark = pytest.mark.gpu

TRACERS = ["while-while", "persistent-while-while", "if-if", "persistent-if-if", "speculative-while-while",
           "persistent-speculative-while-while", "bvh4-speculative-while-while",
           "persistent-bvh4-speculative-while-while"]


@pytest.fixture(autouse=True)
def _needs_cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _dev(a, dtype):
    """A CUDA copy; uint32 arrays travel as int32 (same bits)."""
    import torch
    a = np.ascontiguousarray(a, dtype)
    if a.dtype == np.uint32:
        a = a.view(np.int32)
    return torch.from_numpy(a).cuda()


def _trace(rt, rays_np, any_hit):
    import torch
    rays = _dev(rays_np, np.float32)
    hits = torch.zeros((rays.shape[0], 4), dtype=torch.float32, device="cuda")
    rt.trace(rays, hits, any_hit, torch.cuda.current_stream().cuda_stream)
    rt.check(torch.cuda.current_stream().cuda_stream, timeout_ms=60000)
    return hits.cpu().numpy()


def _occluded(h):
    return (h.view(np.uint32)[:, 3] == 0xFFFFFFFF).astype(np.uint8)


@pytest.fixture(scope="module")
def oracles(orc, golden_scenes):
    return {name: orc.OracleBVH(v, t) for name, (v, t, _, _) in golden_scenes.items()}


@pytest.fixture(params=["sah", "ploc", "lbvh"])
def builder(request, gpu_tracer):
    gpu_tracer.set_device_builder(request.param)
    yield request.param
    gpu_tracer.set_device_builder("default")


@pytest.mark.parametrize("max_tris", [1, 4, 16])
@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_gpu_tree_hits_match_oracle(gpu_tracer, golden_scenes, oracles, name, max_tris, builder):
    v, t, rays, any_rays = golden_scenes[name]
    info = gpu_tracer.build_device(_dev(v, np.float32), _dev(t, np.uint32), max_tris=max_tris)
    assert info["tri_records"] == t.shape[0] and info["depth"] <= 64
    o = oracles[name]
    want, _ = o.closest(rays)
    want_any, _ = o.any(any_rays)
    for tracer in TRACERS:
        gpu_tracer.select(tracer)
        assert_hits_match(_trace(gpu_tracer, rays, False), want, False, f"{name} {tracer} leaf<={max_tris}")
        assert (_occluded(_trace(gpu_tracer, any_rays, True)) == want_any).all(), (name, tracer)
    gpu_tracer.select("while-while")


def test_gpu_tree_spheres_full_frame(gpu_tracer, wl, orc, builder):
    sc, rays = wl.spheres_primary(res=1024)
    info = gpu_tracer.build_device(_dev(sc.vpos, np.float32), _dev(sc.tris, np.uint32), max_tris=4)
    assert info["inner_nodes"] > 0
    want, _ = orc.OracleBVH(sc.vpos, sc.tris).closest(rays)
    for tracer in ("persistent-speculative-while-while", "while-while", "persistent-bvh4-speculative-while-while"):
        gpu_tracer.select(tracer)
        assert_hits_match(_trace(gpu_tracer, rays, False), want, False, f"spheres {tracer}")
    gpu_tracer.select("while-while")


def test_gpu_tree_degenerate_inputs(gpu_tracer, api, builder):
    import torch
    ray = np.array([[0.2, 0.2, 1.0, 1e-4, 0.0, 0.0, -1.0, 3e38]], np.float32)
    tri = np.array([[0, 1, 2, 7]], np.uint32)
    v = np.array([[0, 0, 0, 0], [1, 0, 0, 0], [0, 1, 0, 0]], np.float32)
    # one triangle: the root is a leaf
    gpu_tracer.build_device(_dev(v, np.float32), _dev(tri, np.uint32))
    for tracer in TRACERS:
        gpu_tracer.select(tracer)
        h = _trace(gpu_tracer, ray, False)
        assert h[0, 0] == np.float32(1.0) and h.view(np.uint32)[0, 3] == 0
    # no triangles: every ray misses
    gpu_tracer.build_device(_dev(v, np.float32), torch.zeros((0, 4), dtype=torch.int32, device="cuda"))
    for tracer in TRACERS:
        gpu_tracer.select(tracer)
        h = _trace(gpu_tracer, ray, False)
        assert h[0, 0] == np.float32(3.4028234663852886e38)
    # 5,000 copies of one triangle: equal Morton codes everywhere, equal t for every ray
    many = np.tile(tri, (5000, 1))
    gpu_tracer.build_device(_dev(v, np.float32), _dev(many, np.uint32), max_tris=3)
    for tracer in TRACERS:
        gpu_tracer.select(tracer)
        h = _trace(gpu_tracer, ray, False)
        assert h[0, 0] == np.float32(1.0) and h.view(np.uint32)[0, 3] < 5000
    gpu_tracer.select("while-while")


def test_gpu_tree_nan_vertices(gpu_tracer, wl, orc, builder):
    """Triangles with NaN vertex coordinates (which the host builder refuses) go into the tree
    without an error or an endless build, and are never hit; every other hit equals the
    oracle's on the finite triangles alone, up to near-ties."""
    sc = wl.soup(77, 3000, sigma=0.5)
    lo, hi = sc.bounds()
    rays = wl.shell_rays(78, lo, hi, 20000)
    nv = sc.vpos.shape[0]
    nan_v = np.array([[np.nan, 0, 0, 0], [0, np.nan, 0, 0], [np.nan, np.nan, np.nan, 0]], np.float32)
    v = np.concatenate([sc.vpos, nan_v])
    bad = []
    for k in range(30):  # one, two or three NaN vertices
        good = [int(x) for x in sc.tris[(7 * k) % sc.tris.shape[0], :3]]
        cut = 1 + k % 3
        bad.append([nv + (k + j) % 3 if j < cut else good[j] for j in range(3)] + [0])
    t = np.concatenate([sc.tris, np.array(bad, np.uint32)])
    info = gpu_tracer.build_device(_dev(v, np.float32), _dev(t, np.uint32), max_tris=2)
    assert info["tri_records"] == t.shape[0]
    want, _ = orc.OracleBVH(sc.vpos, sc.tris).closest(rays)
    want_any, _ = orc.OracleBVH(sc.vpos, sc.tris).any(rays)
    for tracer in ("while-while", "persistent-speculative-while-while"):
        gpu_tracer.select(tracer)
        got = _trace(gpu_tracer, rays, False)
        assert (got.view(np.uint32)[:, 3] < sc.tris.shape[0]).all(), "a NaN triangle was hit"
        assert_hits_match(got, want, False, f"NaN vertices, {tracer}")
        assert (_occluded(_trace(gpu_tracer, rays, True)) == want_any).all(), tracer
    gpu_tracer.select("while-while")


def test_gpu_trees_are_deterministic(api, wl, builder):
    """The same scene built twice, and built as one scene of a set whose scenes are built
    concurrently on several host threads, gives the same tree: every closest hit bit for bit."""
    import torch
    sc = wl.soup(91, 40000, sigma=0.5)
    lo, hi = sc.bounds()
    rays = wl.shell_rays(92, lo, hi, 30000)
    v, t = _dev(sc.vpos, np.float32), _dev(sc.tris, np.uint32)
    got = []
    for _ in range(2):
        rt = api.BatchRayTracer(0)
        rt.set_device_builder(builder)
        rt.build_device(v, t, max_tris=2)
        rt.select("while-while")
        got.append(_trace(rt, rays, False))
        rt.close()
    assert (got[0].view(np.uint32) == got[1].view(np.uint32)).all()
    others = [wl.soup(93 + i, 5000 + 3000 * i, sigma=0.5) for i in range(6)]
    scenes = [(_dev(o.vpos, np.float32), _dev(o.tris, np.uint32)) for o in others[:3]] + [(v, t)] + \
             [(_dev(o.vpos, np.float32), _dev(o.tris, np.uint32)) for o in others[3:]]
    rt = api.BatchRayTracer(0)
    rt.set_device_builder(builder)
    rt.build_scenes_device(scenes, max_tris=2)
    rt.select("persistent-while-while")
    d = _dev(rays, np.float32)
    out = torch.zeros((rays.shape[0], 4), device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rt.trace_multi([(3, d, out)], any_hit=False, stream=stream)
    rt.check(stream, timeout_ms=60000)
    assert (out.cpu().numpy().view(np.uint32) == got[0].view(np.uint32)).all()
    rt.close()


def test_sah_scene_set_trees_equal_single_builds(api, wl):
    """With the SAH method the trees of a scene set are built together, one chain of launches
    for the large nodes of every scene, and each scene still gets the tree it gets alone: scenes
    of 0 and 1 triangles, of 2 to 32 (the warp-per-node phase only), just above that, one with a
    NaN vertex, and larger soups. Same statistics, every closest hit bit for bit, the same
    any-hit answers."""
    import torch
    sizes = [5000, 0, 1, 2, 3, 31, 32, 33, 64, 257, 40000, 0, 1, 1000, 70000]
    meshes, rays = [], []
    for i, n in enumerate(sizes):
        if n == 0:
            v, t = np.zeros((3, 4), np.float32), np.zeros((0, 4), np.uint32)
            lo, hi = np.zeros(3, np.float32), np.ones(3, np.float32)
        else:
            sc = wl.soup(400 + i, n, sigma=0.5)
            lo, hi = sc.bounds()
            v, t = sc.vpos.copy(), sc.tris
        if n == 257:
            v[5, 1] = np.nan  # a triangle that no ray hits
        meshes.append((_dev(v, np.float32), _dev(t, np.uint32)))
        rays.append(wl.shell_rays(500 + i, lo, hi, 3000))
    single = []
    rt = api.BatchRayTracer(0)
    rt.select("while-while")
    for (v, t), r in zip(meshes, rays):
        st = rt.build_device(v, t, max_tris=2)
        single.append((st, _trace(rt, r, False), _occluded(_trace(rt, r, True))))
    rt.close()
    rt = api.BatchRayTracer(0)
    stats = rt.build_scenes_device(meshes, max_tris=2)
    rt.select("persistent-while-while")
    stream = torch.cuda.current_stream().cuda_stream
    d = [_dev(r, np.float32) for r in rays]
    for i, (st, _, _) in enumerate(single):
        assert (stats[i]["inner_nodes"], stats[i]["depth"], stats[i]["tri_records"]) == \
            (st["inner_nodes"], st["depth"], st["tri_records"]), i
    for any_hit in (False, True):
        outs = [torch.zeros((r.shape[0], 4), device="cuda") for r in rays]
        rt.trace_multi([(i, d[i], outs[i]) for i in range(len(rays))], any_hit=any_hit, stream=stream)
        rt.check(stream, timeout_ms=60000)
        for i, o in enumerate(outs):
            got = o.cpu().numpy()
            if any_hit:
                assert (_occluded(got) == single[i][2]).all(), i
            else:
                assert (got.view(np.uint32) == single[i][1].view(np.uint32)).all(), i
    rt.close()


def test_gpu_tree_errors(gpu_tracer, api):
    import torch
    v = _dev(np.zeros((3, 4)), np.float32)
    bad = _dev(np.array([[0, 1, 3, 0]]), np.uint32)
    with pytest.raises(api.GRTError) as e:
        gpu_tracer.build_device(v, bad)
    assert e.value.status == 1  # invalid argument: index beyond the vertex count
    with pytest.raises(api.GRTError):
        gpu_tracer.build_device(v, _dev(np.array([[0, 1, 2, 0]]), np.uint32), max_tris=17)
    gpu_tracer.build_device(v, _dev(np.array([[0, 1, 2, 0]]), np.uint32))
    with pytest.raises(api.GRTError):
        gpu_tracer.export_bvh()
    with pytest.raises(ValueError):
        gpu_tracer.build_device(torch.zeros((3, 3), device="cuda"), _dev(np.array([[0, 1, 2, 0]]), np.uint32))
    with pytest.raises(KeyError):
        gpu_tracer.set_device_builder("octree")
    assert api.lib().grt_set_device_builder(gpu_tracer.ctx, 7) == 1  # invalid argument
    for planes in (0, 257):
        assert api.lib().grt_set_device_sah_planes(gpu_tracer.ctx, planes) == 1


def test_sah_builder_tree_quality_equals_host_tree(api, wl):
    """The GPU SAH builder follows the reference builder's split rule, so its tree is visited like
    the host tree built with the same options: inner nodes and triangle tests per bounce ray
    (counted in the exact while-while order over 200,000 diffuse paths of the sphere scene)
    within 3 % of the host tree's, and the same depth up to 2 levels."""
    import torch
    sc, rays = wl.spheres_primary(res=512)
    d_rays = _dev(rays, np.float32)
    counts = {}
    for form in ("host", "sah"):
        rt = api.BatchRayTracer(0)
        if form == "host":
            info = rt.build(sc.vpos, sc.tris, max_tris=2, planes=256, esc=False)
        else:
            rt.set_device_builder("sah", planes=256)
            info = rt.build_device(_dev(sc.vpos, np.float32), _dev(sc.tris, np.uint32), max_tris=2)
        rt.select("while-while")
        hits = torch.zeros((rays.shape[0], 4), device="cuda")
        stream = torch.cuda.current_stream().cuda_stream
        rt.trace(d_rays, hits, False, stream)
        cnt = torch.zeros(3, dtype=torch.int64, device="cuda")
        res = torch.zeros((200_000, 4), dtype=torch.int32, device="cuda")
        rt.set_traversal_counters(cnt)
        rt.pathtrace(api.BatchRayTracer.pt_params(mode=0, seed=5), d_rays, hits, 200_000, res, None, stream)
        rt.check(stream, timeout_ms=60000)
        rt.set_traversal_counters(None)
        c = [int(x) for x in cnt.cpu().numpy()]
        counts[form] = (c[1] / c[0], c[2] / c[0], info["depth"])
        rt.close()
    (hn, ht, hd), (gn, gt, gd) = counts["host"], counts["sah"]
    print(f"per bounce ray: host {hn:.2f} nodes {ht:.2f} tris depth {hd}; GPU SAH {gn:.2f} nodes {gt:.2f} tris depth {gd}")
    assert abs(gn - hn) <= 0.03 * hn and abs(gt - ht) <= 0.03 * ht and abs(gd - hd) <= 2


@pytest.mark.parametrize("set_builder", ["default", "ploc", "lbvh"])
@pytest.mark.parametrize("tracer", ["persistent-while-while", "persistent-speculative-while-while",
                                    "persistent-bvh4-speculative-while-while"])
def test_gpu_scene_set_matches_oracle(api, orc, wl, tracer, set_builder):
    import torch
    rt = api.BatchRayTracer(0)
    rt.set_device_builder(set_builder)
    scenes, rays, oracles = [], [], []
    for i in range(10):
        ntri = wl.log_uniform(93, 2 * i, 1024, 1 << 16)
        nray = wl.log_uniform(93, 2 * i + 1, 4096, 1 << 15)
        sc = wl.soup(300 + i, ntri, sigma=0.5)
        lo, hi = sc.bounds()
        scenes.append((_dev(sc.vpos, np.float32), _dev(sc.tris, np.uint32)))
        r = wl.shell_rays(400 + i, lo, hi, nray)
        r[: nray // 2, 7] = 1.5  # half the rays with a finite t_max
        rays.append(r)
        oracles.append(orc.OracleBVH(sc.vpos, sc.tris))
    scenes.append((_dev(np.zeros((3, 4)), np.float32), torch.zeros((0, 4), dtype=torch.int32, device="cuda")))
    rays.append(rays[0][:64].copy())
    oracles.append(None)
    stats = rt.build_scenes_device(scenes, max_tris=4)
    assert [s["tri_records"] for s in stats] == [int(s[1].shape[0]) for s in scenes]
    with pytest.raises(api.GRTError):
        rt.export_scene_bvh(0, 1, 1)
    rt.select(tracer)
    stream = torch.cuda.current_stream().cuda_stream
    for any_hit in (False, True):
        d_rays = [_dev(r, np.float32) for r in rays]
        outs = [torch.zeros((r.shape[0], 4), device="cuda") for r in rays]
        rt.trace_multi([(s, d_rays[s], outs[s]) for s in range(len(rays))], any_hit=any_hit, stream=stream)
        rt.check(stream, timeout_ms=60000)
        for s, o in enumerate(oracles):
            got = outs[s].cpu().numpy()
            if o is None:
                assert (got[:, 0] == np.float32(3.4028234663852886e38)).all()
            elif any_hit:
                assert (_occluded(got) == o.any(rays[s])[0]).all(), (tracer, s)
            else:
                assert_hits_match(got, o.closest(rays[s])[0], False, f"{tracer} scene {s}")
    rt.close()
