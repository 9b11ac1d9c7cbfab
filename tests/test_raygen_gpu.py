"""The incoherent test rays of `incoherence r1 r2` (grt_incoherent_rays; the reference's
setup_ray_incoherent, rt/cuda/kernels.cu:75-156, with the sphere placement of
rt/cuda/rni.cpp:36-66): every ray starts in the first ball and aims into the second, the balls
sit where the reference places them, the samples are uniform in the balls, the stream is
reproducible per seed, and the rays trace like any others."""
import numpy as np
import pytest

from conftest import assert_hits_match

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _needs_cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def placement(vpos):
    """The reference's sphere placement over the scene's vertex extent (rni.cpp:38-66)."""
    lo = vpos[:, :3].min(0).astype(np.float64)
    hi = vpos[:, :3].max(0).astype(np.float64)
    sx, sy, sz = size = np.abs(hi - lo)
    axis = 0 if sx >= sy and sx >= sz else (1 if sy >= sx and sy >= sz else 2)
    r_max = size[axis] / 4
    c1 = lo + size / 2
    c2 = c1.copy()
    c1[axis] = lo[axis] + r_max
    c2[axis] = hi[axis] - r_max
    return c1, c2, r_max


@pytest.fixture(scope="module")
def scene_rt(api, wl):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    sc = wl.spheres()
    rt = api.BatchRayTracer(0)
    rt.build(sc.vpos, sc.tris)
    yield sc, rt
    rt.close()


def test_rays_start_in_the_first_ball_and_aim_into_the_second(scene_rt):
    sc, rt = scene_rt
    c1, c2, r_max = placement(sc.vpos)
    rays = rt.incoherent_rays(200000, seed=7, r1=0.5, r2=0.25).cpu().numpy().astype(np.float64)
    o, d = rays[:, 0:3], rays[:, 4:7]
    assert (rays[:, 3] == 0).all() and (rays[:, 7] == np.float32(3.4028234663852886e38)).all()
    assert np.allclose(np.linalg.norm(d, axis=1), 1.0, atol=1e-6)
    r_o = np.linalg.norm(o - c1, axis=1) / (0.5 * r_max)
    assert r_o.max() <= 1 + 1e-5
    # uniform in the ball: P(r < R/2) = 1/8, the mean offset is the centre
    assert abs((r_o < 0.5).mean() - 0.125) < 0.005
    assert np.abs((o - c1).mean(0)).max() < 0.01 * r_max
    # the ray passes within r2 * r_max of the second centre
    w = c2 - o
    dist = np.linalg.norm(w - (w * d).sum(1, keepdims=True) * d, axis=1)
    assert dist.max() <= 0.25 * r_max * (1 + 1e-4) + 1e-4


def test_zero_radii_give_the_centre_to_centre_ray_and_seeds_repeat(scene_rt):
    import torch
    sc, rt = scene_rt
    c1, c2, _ = placement(sc.vpos)
    rays = rt.incoherent_rays(1000, r1=0.0, r2=0.0).cpu().numpy()
    assert np.allclose(rays[:, 0:3], c1, atol=1e-5)
    want = (c2 - c1) / np.linalg.norm(c2 - c1)
    assert np.allclose(rays[:, 4:7], want, atol=1e-6)
    assert (rays == rays[0]).all()
    a = rt.incoherent_rays(5000, seed=3, r1=1.0, r2=1.0)
    b = rt.incoherent_rays(5000, seed=3, r1=1.0, r2=1.0)
    c = rt.incoherent_rays(5000, seed=4, r1=1.0, r2=1.0)
    assert torch.equal(a, b) and not torch.equal(a, c)


def test_incoherence_command_and_tracing(api, orc, scene_rt):
    sc, rt = scene_rt
    assert rt.interprete("incoherence 0.5 0.5")
    assert rt.use_incoherence and rt.incoherence_r1 == 0.5 and rt.incoherence_r2 == 0.5
    assert rt.interprete("incoherence 0 0") and rt.incoherence_r1 == 0.5  # 0 0 leaves it as it was
    with pytest.raises(ValueError):
        rt.interprete("incoherence -1 0")
    with pytest.raises(ValueError):
        rt.interprete("incoherence 1")
    rays = rt.incoherent_rays(65536, seed=11)
    import torch
    hits = torch.zeros((rays.shape[0], 4), device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rt.select("while-while")
    rt.trace(rays, hits, False, stream)
    rt.check(stream)
    want, _ = orc.OracleBVH(sc.vpos, sc.tris).closest(rays.cpu().numpy())
    assert_hits_match(hits.cpu().numpy(), want, True, "incoherent rays")
    assert (want[:, 0] < 3e38).mean() > 0.1  # the rays cross the sphere field
    with pytest.raises(api.GRTError):
        rt.incoherent_rays(10, r1=-1.0, r2=0.0)
