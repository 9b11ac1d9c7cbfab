"""Direct lighting by light-source sampling (grt_direct: the reference's direct-wf steps) in
the wavefront and the fused persistent form: both equal the oracle's restatement in every bit of
the frame buffer for the exact loop orders, on spheres with a floor and two area lights."""
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
