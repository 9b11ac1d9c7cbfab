"""Direct lighting (grt_direct: the reference's direct-wf steps) by light-source sampling and by
uniform or cosine-weighted direction sampling, in the wavefront and the fused persistent form:
both equal the oracle's restatement in every bit of the frame buffer for the exact loop orders,
on spheres with a floor and two area lights; the three strategies estimate the same light.
Also primary-wf's albedo shading (grt_hit_albedo) in both forms."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _needs_cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


@pytest.fixture(scope="module")
def lit_case(orc, wl):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    sc, mats, rays = wl.lit_spheres(count=48, res=160)
    o = orc.OracleBVH(sc.vpos, sc.tris)
    want = o.direct(rays, mats, samples=3, seed=11)
    return sc, mats, rays, want


@pytest.mark.parametrize("tracer", ["while-while", "persistent-while-while", "if-if", "persistent-if-if"])
@pytest.mark.parametrize("mode", ["wavefront", "fused"])
def test_direct_matches_oracle(api, lit_case, tracer, mode):
    import torch
    sc, mats, rays, want = lit_case
    lit = want[:, :3].sum(1) > 0
    assert lit.mean() > 0.2 and np.isfinite(want).all()  # the lights reach a good part of the frame
    rt = api.BatchRayTracer(0)
    rt.build(sc.vpos, sc.tris)
    rt.set_material_table(mats)
    rt.select(tracer)
    r = torch.from_numpy(rays).cuda()
    fb = torch.zeros((rays.shape[0], 4), device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rt.direct(r, fb, samples=3, mode=api.DL_FUSED if mode == "fused" else api.DL_WAVEFRONT, seed=11, stream=stream)
    rt.check(stream, timeout_ms=60000)
    got = fb.cpu().numpy()
    bad = (got.view(np.uint32) != want.view(np.uint32)).any(1)
    assert not bad.any(), f"{bad.sum()} pixels differ, first {np.nonzero(bad)[0][:5]}"
    rt.close()


@pytest.fixture(scope="module")
def dir_cases(orc, lit_case):
    sc, mats, rays, _ = lit_case
    o = orc.OracleBVH(sc.vpos, sc.tris)
    return {smp: o.direct(rays, mats, samples=3, seed=11, sampling=smp) for smp in ("uniform", "cosine")}


@pytest.mark.parametrize("sampling", ["uniform", "cosine"])
@pytest.mark.parametrize("tracer", ["while-while", "persistent-while-while", "if-if", "persistent-if-if"])
@pytest.mark.parametrize("mode", ["wavefront", "fused"])
def test_direct_direction_sampling_matches_oracle(api, lit_case, dir_cases, tracer, mode, sampling):
    """k::sample_uniform_dir / k::sample_cos_dir, a closest-hit trace, k::integrate_dir."""
    import torch
    sc, mats, rays, _ = lit_case
    want = dir_cases[sampling]
    assert (want[:, :3].sum(1) > 0).mean() > 0.01 and np.isfinite(want).all()
    rt = api.BatchRayTracer(0)
    rt.build(sc.vpos, sc.tris)
    rt.set_material_table(mats)
    rt.select(tracer)
    r = torch.from_numpy(rays).cuda()
    fb = torch.zeros((rays.shape[0], 4), device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rt.direct(r, fb, samples=3, mode=api.DL_FUSED if mode == "fused" else api.DL_WAVEFRONT, seed=11, stream=stream,
              sampling=sampling)
    rt.check(stream, timeout_ms=60000)
    bad = (fb.cpu().numpy().view(np.uint32) != want.view(np.uint32)).any(1)
    assert not bad.any(), f"{bad.sum()} pixels differ, first {np.nonzero(bad)[0][:5]}"
    rt.close()


def test_direct_strategies_estimate_the_same_light(api, lit_case):
    """Light, uniform and cosine sampling are estimators of the same direct light: at 256 samples
    per pixel their means over the pixels that see a non-emitting surface agree within a few
    percent (the one-sidedness of light sampling and the noise of uniform sampling allowed for)."""
    import torch
    sc, mats, rays, _ = lit_case
    rt = api.BatchRayTracer(0)
    rt.build(sc.vpos, sc.tris)
    rt.set_material_table(mats)
    rt.select("persistent-speculative-while-while")
    r = torch.from_numpy(rays).cuda()
    stream = torch.cuda.Stream()
    hits = torch.zeros((rays.shape[0], 4), device="cuda")
    rt.trace(r, hits, False, stream.cuda_stream)
    means = {}
    for smp in ("light", "uniform", "cosine"):
        fb = torch.zeros((rays.shape[0], 4), device="cuda")
        rt.direct(r, fb, samples=256, mode=api.DL_FUSED, seed=5, stream=stream.cuda_stream, sampling=smp)
        rt.check(stream.cuda_stream, timeout_ms=60000)
        means[smp] = fb.cpu().numpy()
    h = hits.cpu().numpy()
    hit = h[:, 0] < 3e38
    ref = h[:, 3].view(np.uint32)
    emits = np.zeros(len(h), bool)
    emits[hit] = mats[sc.tris[ref[hit], 3], 3:6].sum(1) > 0
    sel = hit & ~emits
    assert sel.mean() > 0.3
    m = {k: v[sel, :3].mean() for k, v in means.items()}
    assert all((v[:, 3] == 256).all() for v in means.values())
    assert abs(m["uniform"] / m["light"] - 1) < 0.05 and abs(m["cosine"] / m["light"] - 1) < 0.05, m
    bad = api.DirectParams(1, api.DL_FUSED, 0, 3, 0)  # no such strategy
    fb = torch.zeros((rays.shape[0], 4), device="cuda")
    with pytest.raises(api.GRTError) as e:
        rt._check(api.lib().grt_direct(rt.ctx, ctypes.byref(bad), r.data_ptr(), int(r.shape[0]), fb.data_ptr(),
                                       stream.cuda_stream))
    assert e.value.status == 1
    rt.close()


@pytest.mark.parametrize("tracer", ["while-while", "persistent-while-while", "if-if", "persistent-speculative-while-while"])
@pytest.mark.parametrize("mode", ["wavefront", "fused"])
def test_hit_albedo_matches_oracle(api, orc, lit_case, tracer, mode):
    """primary-wf's shading step, add_hitpoint_albedo: fb += (albedo of the hit, 1), accumulated
    onto what the frame buffer held; one material id beyond the table gets the default (0)."""
    import torch
    sc, mats, rays, _ = lit_case
    tris = sc.tris.copy()
    tris[::97, 3] = mats.shape[0] + 5  # a few triangles with an unknown material
    o = orc.OracleBVH(sc.vpos, tris)
    fb0 = np.random.default_rng(7).random((rays.shape[0], 4), dtype=np.float32)
    want = o.hit_albedo(rays, mats, fb0)
    rt = api.BatchRayTracer(0)
    rt.build(sc.vpos, tris)
    rt.set_material_table(mats)
    rt.select(tracer)
    r = torch.from_numpy(rays).cuda()
    fb = torch.from_numpy(fb0.copy()).cuda()
    stream = torch.cuda.current_stream().cuda_stream
    rt.hit_albedo(r, fb, mode=api.DL_FUSED if mode == "fused" else api.DL_WAVEFRONT, stream=stream)
    rt.check(stream, timeout_ms=60000)
    got = fb.cpu().numpy()
    bad = (got.view(np.uint32) != want.view(np.uint32)).any(1)
    if "speculative" in tracer:  # the other triangle of a near-tie may carry another albedo
        assert bad.mean() < 1e-3, int(bad.sum())
    else:
        assert not bad.any(), f"{bad.sum()} pixels differ, first {np.nonzero(bad)[0][:5]}"
    assert (got[:, 3] == fb0[:, 3] + 1).all()
    rt.close()


@pytest.mark.parametrize("tracer", ["speculative-while-while", "persistent-bvh4-speculative-while-while"])
def test_direct_speculative_orders(api, lit_case, tracer):
    """The speculative orders may pick the other triangle of a near-tie for a camera ray; every
    other pixel is bit-identical to the oracle."""
    import torch
    sc, mats, rays, want = lit_case
    rt = api.BatchRayTracer(0)
    rt.build(sc.vpos, sc.tris)
    rt.set_material_table(mats)
    rt.select(tracer)
    r = torch.from_numpy(rays).cuda()
    stream = torch.cuda.current_stream().cuda_stream
    for mode in (api.DL_FUSED, api.DL_WAVEFRONT):
        fb = torch.zeros((rays.shape[0], 4), device="cuda")
        rt.direct(r, fb, samples=3, mode=mode, seed=11, stream=stream)
        rt.check(stream, timeout_ms=60000)
        bad = (fb.cpu().numpy().view(np.uint32) != want.view(np.uint32)).any(1)
        assert bad.mean() < 1e-3, (tracer, mode, int(bad.sum()))
    rt.close()


def test_direct_accumulates_and_checks_inputs(api, lit_case):
    import torch
    sc, mats, rays, want = lit_case
    rt = api.BatchRayTracer(0)
    r = torch.from_numpy(rays).cuda()
    fb = torch.zeros((rays.shape[0], 4), device="cuda")
    with pytest.raises(api.GRTError):
        rt.set_material_table(mats)  # before a build
    rt.build(sc.vpos, sc.tris)
    with pytest.raises(api.GRTError):
        rt.direct(r, fb, samples=1)  # no material table
    rt.set_material_table(mats)
    stream = torch.cuda.current_stream().cuda_stream
    # two calls of 3 samples each with the same seed add the same values twice
    rt.direct(r, fb, samples=3, mode=api.DL_FUSED, seed=11, stream=stream)
    rt.direct(r, fb, samples=3, mode=api.DL_WAVEFRONT, seed=11, stream=stream)
    rt.check(stream)
    got = fb.cpu().numpy()
    assert (got[:, 3] == 6).all()
    assert np.allclose(got[:, :3], 2 * want[:, :3], rtol=1e-6, atol=0)
    rt.close()
