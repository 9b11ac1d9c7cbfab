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


def _golden_camera():
    import os
    return dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "golden_camera.npz")))


def test_camera_rays_equal_reference_cam_ray(api, orc):
    """grt_camera_rays against the reference's own cam_ray (golden cases: pixel centres, PCG
    jitter, explicit offsets) and against the oracle's restatement at 1024x1024 and 1920x1080,
    bit for bit."""
    import torch
    from make_golden_camera import camera_cases
    g = _golden_camera()
    rt = api.BatchRayTracer(0)
    for name, pos, d, up, nw, nh, w, h, mode, seed, _ in camera_cases():
        off = g.get(name + "/offsets")
        d_off = torch.from_numpy(off).cuda() if off is not None else None
        rays = rt.camera_rays(pos, d, up, nw, nh, w, h, offsets=d_off, jitter=mode == "jitter", seed=seed)
        torch.cuda.synchronize()
        assert (rays.cpu().numpy().view(np.uint32) == g[name + "/rays"].view(np.uint32)).all(), name
    d = np.array((0.0, 0.0, -1.0), np.float32)
    for w, h, jitter in ((1024, 1024, True), (1920, 1080, False)):
        rays = rt.camera_rays((0.0, 0.0, 35.0), d, (0.0, 1.0, 0.0), 0.6370703 * w / h, 0.6370703, w, h,
                              jitter=jitter, seed=5)
        torch.cuda.synchronize()
        want = orc.cam_rays((0.0, 0.0, 35.0), d, (0.0, 1.0, 0.0), 0.6370703 * w / h, 0.6370703, w, h, None, jitter, 5)
        assert (rays.cpu().numpy().view(np.uint32) == want.view(np.uint32)).all(), (w, h)
    rt.close()


def test_camera_rays_arguments(api):
    import torch
    rt = api.BatchRayTracer(0)
    ok = torch.zeros((16, 8), device="cuda")
    cam = ((0.0, 0.0, 5.0), (0.0, 0.0, -1.0), (0.0, 1.0, 0.0), 0.5, 0.5)
    rt.camera_rays(*cam, 4, 4, rays=ok)
    with pytest.raises(ValueError):
        rt.camera_rays(*cam, 5, 4, rays=ok)  # too small
    raw = torch.zeros(16 * 8 + 1, device="cuda")
    with pytest.raises(api.GRTError):
        rt.camera_rays(*cam, 4, 4, rays=raw[1:].view(16, 8))  # misaligned
    rt.camera_rays(*cam, 0, 4, rays=ok)  # no pixels: nothing to do
    rt.close()
