"""Alpha-aware tracing (the "<tracer>-alpha" names, grt_set_alpha) against the reference's
alpha-aware CPU tracer (golden_alpha.npz, from binary_bvh_tracer<indexed, esc on, true>) and
the oracle's alpha restatement: exact tracers bit-identical, speculative ones up to near-ties,
any-hit answers equal; diffuse paths through the alpha tracer equal the oracle's in every word."""
import numpy as np
import pytest

import cases
from conftest import assert_hits_match, load_golden

pytestmark = pytest.mark.gpu

BASE = ["while-while", "persistent-while-while", "if-if", "persistent-if-if", "speculative-while-while",
        "persistent-speculative-while-while", "bvh4-speculative-while-while",
        "persistent-bvh4-speculative-while-while"]


@pytest.fixture(autouse=True)
def _needs_cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _trace(rt, rays_np, any_hit):
    import torch
    rays = torch.from_numpy(np.ascontiguousarray(rays_np, np.float32)).cuda()
    hits = torch.zeros((rays.shape[0], 4), dtype=torch.float32, device="cuda")
    rt.trace(rays, hits, any_hit, torch.cuda.current_stream().cuda_stream)
    rt.check(torch.cuda.current_stream().cuda_stream, timeout_ms=60000)
    return hits.cpu().numpy()


def _occluded(h):
    return (h.view(np.uint32)[:, 3] == 0xFFFFFFFF).astype(np.uint8)


@pytest.fixture(scope="module")
def alpha_case():
    v, t, tc, mat_tex, textures = cases.alpha_scene()
    rays, any_rays = cases.alpha_rays()
    return dict(v=v, t=t, tc=tc, mat_tex=mat_tex, textures=textures, rays=rays, any_rays=any_rays,
                g=load_golden("alpha"))


@pytest.mark.parametrize("tracer", BASE)
def test_alpha_tracers_match_reference(gpu_tracer, alpha_case, tracer):
    c = alpha_case
    gpu_tracer.build(c["v"], c["t"])
    gpu_tracer.set_alpha(c["tc"], c["mat_tex"], c["textures"])
    gpu_tracer.select(tracer + "-alpha")
    exact = "speculative" not in tracer
    assert_hits_match(_trace(gpu_tracer, c["rays"], False), c["g"]["closest"], exact, tracer + "-alpha")
    assert (_occluded(_trace(gpu_tracer, c["any_rays"], True)) == c["g"]["any_occluded"]).all()
    # the same tracer without "-alpha" ignores the texture data
    gpu_tracer.select(tracer)
    plain = _trace(gpu_tracer, c["rays"], False)
    assert (plain.view(np.uint32) != c["g"]["closest"].view(np.uint32)).any()
    gpu_tracer.select("while-while")


def test_alpha_tracer_without_texture_data_is_opaque(gpu_tracer, alpha_case, orc):
    c = alpha_case
    gpu_tracer.build(c["v"], c["t"])
    gpu_tracer.select("persistent-while-while-alpha")
    want, _ = orc.OracleBVH(c["v"], c["t"]).closest(c["rays"])
    assert_hits_match(_trace(gpu_tracer, c["rays"], False), want, True, "no texture data")
    gpu_tracer.select("while-while")


def test_alpha_on_gpu_built_tree(gpu_tracer, alpha_case):
    import torch
    c = alpha_case
    gpu_tracer.build_device(torch.from_numpy(c["v"]).cuda(), torch.from_numpy(c["t"].view(np.int32)).cuda())
    gpu_tracer.set_alpha(c["tc"], c["mat_tex"], c["textures"])
    for tracer in ("persistent-speculative-while-while-alpha", "while-while-alpha"):
        gpu_tracer.select(tracer)
        assert_hits_match(_trace(gpu_tracer, c["rays"], False), c["g"]["closest"], False, tracer)
        assert (_occluded(_trace(gpu_tracer, c["any_rays"], True)) == c["g"]["any_occluded"]).all()
    gpu_tracer.select("while-while")


@pytest.mark.parametrize("mode", ["wavefront", "fused"])
def test_alpha_paths_match_oracle(api, orc, alpha_case, mode):
    """Diffuse paths bouncing between the two textured grids, traced by an exact alpha tracer,
    equal the oracle's alpha-aware path tracer in every result word and bounce hit."""
    import torch
    c = alpha_case
    o = orc.OracleBVH(c["v"], c["t"])
    o.set_alpha(orc.AlphaSet(c["tc"], c["mat_tex"], c["textures"]))
    prim = c["rays"][: 96 * 96]
    prim_hits, _ = o.closest(prim)
    n_paths = 40000
    want, want_b = o.pathtrace(prim, prim_hits, n_paths, bounce_hits=True)
    rt = api.BatchRayTracer(0)
    rt.build(c["v"], c["t"])
    rt.set_alpha(c["tc"], c["mat_tex"], c["textures"])
    rt.select("persistent-while-while-alpha" if mode == "fused" else "while-while-alpha")
    rays = torch.from_numpy(prim).cuda()
    hits = torch.from_numpy(prim_hits).cuda()
    res = torch.zeros((n_paths, 4), dtype=torch.int32, device="cuda")
    bh = torch.zeros((n_paths, 5, 4), dtype=torch.float32, device="cuda")
    p = api.BatchRayTracer.pt_params(mode=api.PT_FUSED if mode == "fused" else api.PT_WAVEFRONT)
    stream = torch.cuda.current_stream().cuda_stream
    rt.pathtrace(p, rays, hits, n_paths, res, bh, stream)
    rt.check(stream, timeout_ms=60000)
    assert (res.cpu().numpy().view(np.uint32) == want).all()
    assert (bh.cpu().numpy().view(np.uint32) == want_b.view(np.uint32)).all()
    rt.close()


def test_alpha_errors(api, alpha_case):
    import torch
    c = alpha_case
    rt = api.BatchRayTracer(0)
    with pytest.raises(api.GRTError) as e:
        rt.set_alpha(c["tc"], c["mat_tex"], c["textures"])
    assert e.value.status == 6  # before a build
    rt.build(c["v"], c["t"])
    with pytest.raises(api.GRTError):
        rt.set_alpha(c["tc"][:-1], c["mat_tex"], c["textures"])  # one vertex short
    with pytest.raises(api.GRTError):
        rt.set_alpha(c["tc"], np.array([-1, 5], np.int32), c["textures"])  # no texture 5
    rt.set_alpha(c["tc"], c["mat_tex"], c["textures"])
    rt.set_alpha(None, None, None)  # cleared
    rt.build_scenes([(c["v"], c["t"])])
    rt.select("persistent-while-while-alpha")
    r = torch.from_numpy(c["rays"][:64]).cuda()
    h = torch.zeros((64, 4), device="cuda")
    with pytest.raises(api.GRTError):
        rt.trace_multi([(0, r, h)])
    rt.close()
