"""GPU parity: the sm_103a kernels, called through the C-ABI, return exactly the reference's
closest hits (triangle, t, beta, gamma bit for bit) and any-hit answers."""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, assert_hits_match, load_golden, same_bits

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _needs_cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")

TRACERS = ["while-while", "persistent-while-while", "if-if", "persistent-if-if", "speculative-while-while",
           "persistent-speculative-while-while", "bvh4-speculative-while-while",
           "persistent-bvh4-speculative-while-while"]


def exact(tracer):
    return "speculative" not in tracer


def _trace(rt, rays_np, any_hit):
    import torch
    rays = torch.from_numpy(np.ascontiguousarray(rays_np, np.float32)).cuda()
    hits = torch.zeros((rays.shape[0], 4), dtype=torch.float32, device="cuda")
    rt.trace(rays, hits, any_hit, torch.cuda.current_stream().cuda_stream)
    rt.check(torch.cuda.current_stream().cuda_stream, timeout_ms=60000)
    return hits.cpu().numpy()


def occluded(h):
    return (h.view(np.uint32)[:, 3] == 0xFFFFFFFF).astype(np.uint8)


@pytest.mark.parametrize("tracer", TRACERS)
@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_golden_closest_and_any(gpu_tracer, golden_scenes, name, tracer):
    g = load_golden(name)
    v, t, rays, any_rays = golden_scenes[name]
    gpu_tracer.build(v, t)
    gpu_tracer.select(tracer)
    got = _trace(gpu_tracer, rays, False)
    assert_hits_match(got, g["closest"], exact(tracer), f"{name} closest hits")
    got_any = _trace(gpu_tracer, any_rays, True)
    assert (occluded(got_any) == g["any_occluded"]).all()
    t_bits = got_any.view(np.uint32)[:, 0]
    assert (t_bits[g["any_occluded"] == 1] == np.float32(4294967296.0).view(np.uint32)).all()
    assert (got_any[g["any_occluded"] == 0, 0] == np.float32(3.4028234663852886e38)).all()


@pytest.mark.parametrize("tracer", TRACERS)
def test_spheres_primary_1024_matches_oracle(gpu_tracer, orc, wl, tracer):
    sc, rays = wl.spheres_primary()
    o = orc.OracleBVH(sc.vpos, sc.tris)
    want, cnt = o.closest(rays, counts=True)
    gpu_tracer.build(sc.vpos, sc.tris)
    gpu_tracer.select(tracer)
    got = _trace(gpu_tracer, rays, False)
    assert_hits_match(got, want, exact(tracer))
    assert int(cnt[:, 2].max()) <= 24


@pytest.mark.parametrize("builder", [dict(split="sah", max_tris=1, esc=False), dict(split="om", max_tris=8),
                                     dict(split="sm", max_tris=16, esc=False)])
def test_other_builders_match_oracle(gpu_tracer, orc, wl, builder):
    sc = wl.soup(31, 20000)
    lo, hi = sc.bounds()
    rays = wl.shell_rays(32, lo, hi, 50000)
    o = orc.OracleBVH(sc.vpos, sc.tris, planes=16, **builder)
    gpu_tracer.build(sc.vpos, sc.tris, planes=16, **builder)
    for tracer in TRACERS:
        gpu_tracer.select(tracer)
        assert_hits_match(_trace(gpu_tracer, rays, False), o.closest(rays)[0], exact(tracer))
        r2 = rays.copy()
        r2[:, 7] = 2.0
        assert (occluded(_trace(gpu_tracer, r2, True)) == o.any(r2)[0]).all()


@pytest.mark.parametrize("tracer", TRACERS)
def test_tuned_tree_spheres_matches_oracle(gpu_tracer, orc, wl, tracer):
    """The benchmark's tuned tree (leaves of at most 2, 64 SAH planes, no clipping) on the
    1024x1024 sphere frame, closest and any hit."""
    sc, rays = wl.spheres_primary()
    opts = dict(split="sah", max_tris=2, planes=64, esc=False)
    o = orc.OracleBVH(sc.vpos, sc.tris, **opts)
    gpu_tracer.build(sc.vpos, sc.tris, **opts)
    gpu_tracer.select(tracer)
    assert_hits_match(_trace(gpu_tracer, rays, False), o.closest(rays)[0], exact(tracer))
    r2 = rays[::16].copy()
    r2[:, 7] = 5.0
    assert (occluded(_trace(gpu_tracer, r2, True)) == o.any(r2)[0]).all()


def test_trace_host_path_matches(gpu_tracer, wl, orc):
    sc, rays = wl.heightfield_primary()
    gpu_tracer.build(sc.vpos, sc.tris)
    gpu_tracer.select("while-while")
    got = gpu_tracer.trace_host(rays)
    assert same_bits(got, orc.OracleBVH(sc.vpos, sc.tris).closest(rays)[0]).all()


def test_errors_are_status_codes(api, wl):
    import torch
    rt = api.BatchRayTracer(0)
    rays = torch.zeros((4, 8), device="cuda")
    hits = torch.zeros((4, 4), device="cuda")
    with pytest.raises(api.GRTError) as e:
        rt.trace(rays, hits)
    assert e.value.status == 6  # not built
    with pytest.raises(api.GRTError) as e:
        rt.select("no-such-tracer")
    assert e.value.status == 8
    assert rt.interprete("bvh type om") and rt.bvh_type == "om"
    assert not rt.interprete("frobnicate 3")
    sc, _ = wl.heightfield_primary()
    rt.build(sc.vpos, sc.tris)
    raw = torch.zeros(4 * 8 + 1, device="cuda")
    with pytest.raises(api.GRTError) as e:
        rt.trace(raw[1:].view(4, 8), hits)  # misaligned rays
    assert e.value.status == 1
    rt.close()


@pytest.mark.parametrize("alias,same", [("simple", "if-if"), ("dynamic-while-while", "persistent-while-while"),
                                        ("simple-alpha", "if-if-alpha"),
                                        ("dynamic-while-while-alpha", "persistent-while-while-alpha")])
def test_reference_tracer_names(gpu_tracer, golden_scenes, alias, same):
    """Every `raytracer` name of the reference's CUDA platform (rt/cuda/platform.cpp:102-131)
    selects a tracer; `simple` and `dynamic-while-while` give the reference's hits exactly."""
    name = GOLDEN_CASES[0]
    g = load_golden(name)
    v, t, rays, any_rays = golden_scenes[name]
    gpu_tracer.build(v, t)
    assert gpu_tracer.interprete(f"raytracer {alias}")
    got = _trace(gpu_tracer, rays, False)
    assert_hits_match(got, g["closest"], True, f"{alias} closest hits")
    assert (occluded(_trace(gpu_tracer, any_rays, True)) == g["any_occluded"]).all()
    gpu_tracer.select(same)
    assert same_bits(_trace(gpu_tracer, rays, False), got).all()
    gpu_tracer.select("while-while")


def test_empty_scene_misses(gpu_tracer):
    v = np.zeros((3, 4), np.float32)
    gpu_tracer.build(v, np.zeros((0, 4), np.uint32), esc=False)
    rays = np.tile(np.array([[0, 0, 1, 1e-4, 0, 0, -1, 3e38]], np.float32), (100, 1))
    for tracer in TRACERS:
        gpu_tracer.select(tracer)
        got = _trace(gpu_tracer, rays, False)
        assert (got[:, 0] == np.float32(3.4028234663852886e38)).all() and (got.view(np.uint32)[:, 3] == 0).all()
