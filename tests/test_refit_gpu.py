"""Refit (grt_refit): a built tree follows new vertex positions with its topology kept. Refitting
to unchanged vertices gives back the same boxes (traces bit-identical with every tracer, 4-wide
ones included); after the vertices move, closest hits equal the oracle's on the moved mesh up to
near-ties and any-hit answers are equal; the autograd binding refits between steps."""
import numpy as np
import pytest

from conftest import assert_hits_match, same_bits

pytestmark = pytest.mark.gpu

TRACERS = ["while-while", "persistent-while-while", "if-if", "speculative-while-while",
           "persistent-speculative-while-while", "bvh4-speculative-while-while",
           "persistent-bvh4-speculative-while-while"]


@pytest.fixture(autouse=True)
def _needs_cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _dev(a, dtype):
    import torch
    a = np.ascontiguousarray(a, dtype)
    if a.dtype == np.uint32:
        a = a.view(np.int32)
    return torch.from_numpy(a).cuda()


def _trace(rt, rays, any_hit):
    import torch
    hits = torch.zeros((rays.shape[0], 4), device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rt.trace(rays, hits, any_hit, stream)
    rt.check(stream, timeout_ms=60000)
    return hits.cpu().numpy()


def _occluded(h):
    return h.view(np.uint32)[:, 3] == 0xFFFFFFFF


def _moved(v, seed, scale):
    g = np.random.default_rng(seed)
    w = np.array(v, np.float32, copy=True)
    w[:, :3] += (scale * g.normal(size=(w.shape[0], 3))).astype(np.float32)
    return w


@pytest.mark.parametrize("builder", ["host", "gpu"])
def test_refit_to_the_same_vertices_changes_nothing(api, wl, builder):
    sc, rays_np = wl.spheres_primary(res=256)
    lo, hi = sc.bounds()
    rays = _dev(rays_np, np.float32)
    shadow = _dev(wl.shell_rays(9, lo, hi, 20000), np.float32)
    rt = api.BatchRayTracer(0)
    if builder == "host":
        rt.build(sc.vpos, sc.tris, esc=False)  # no clipped boxes: every box is its triangles' bounds
    else:
        rt.build_device(_dev(sc.vpos, np.float32), _dev(sc.tris, np.uint32))
    before = {}
    for tracer in TRACERS:
        rt.select(tracer)
        before[tracer] = (_trace(rt, rays, False), _trace(rt, shadow, True))
    rt.refit(_dev(sc.vpos, np.float32))
    for tracer in TRACERS:
        rt.select(tracer)
        c, a = _trace(rt, rays, False), _trace(rt, shadow, True)
        assert same_bits(c, before[tracer][0]).all(), tracer
        assert same_bits(a, before[tracer][1]).all(), tracer
    rt.close()


@pytest.mark.parametrize("builder", ["host", "gpu"])
def test_refit_follows_moved_vertices(api, wl, orc, builder):
    sc = wl.icosphere(levels=5)
    rays_np = wl.camera_rays((0.0, 0.0, 3.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 50.0, 256, 256)
    rays = _dev(rays_np, np.float32)
    lo, hi = sc.bounds()
    rt = api.BatchRayTracer(0)
    if builder == "host":
        rt.build(sc.vpos, sc.tris)  # with early split clipping: refit replaces the clipped boxes
    else:
        rt.build_device(_dev(sc.vpos, np.float32), _dev(sc.tris, np.uint32))
    v = sc.vpos
    for step in range(3):
        v = _moved(v, 20 + step, 0.01)
        rt.refit(_dev(v, np.float32))
        o = orc.OracleBVH(v, sc.tris)
        want, _ = o.closest(rays_np)
        shadow_np = wl.shell_rays(30 + step, lo, hi, 20000)
        shadow_np[:, 7] = 1.0
        want_any, _ = o.any(shadow_np)
        for tracer in ("while-while", "persistent-speculative-while-while", "persistent-bvh4-speculative-while-while"):
            rt.select(tracer)
            assert_hits_match(_trace(rt, rays, False), want, False, f"{builder} step {step} {tracer}")
            assert (_occluded(_trace(rt, _dev(shadow_np, np.float32), True)) == want_any.astype(bool)).all()
    rt.close()


def test_refit_errors(api, wl):
    import torch
    sc, _ = wl.spheres_primary(res=64)
    rt = api.BatchRayTracer(0)
    v = _dev(sc.vpos, np.float32)
    with pytest.raises(api.GRTError) as e:
        rt.refit(v)
    assert e.value.status == 6  # not built
    rt.build(sc.vpos, sc.tris)
    rt.export_bvh()
    with pytest.raises(api.GRTError) as e:
        rt.refit(v[:-1].contiguous())
    assert e.value.status == 1  # another vertex count
    raw = torch.zeros(v.numel() + 1, device="cuda")
    with pytest.raises(api.GRTError) as e:
        rt.refit(raw[1:].view(-1, 4))  # misaligned
    assert e.value.status == 1
    rt.refit(v)
    with pytest.raises(api.GRTError):
        rt.export_bvh()  # the refitted tree is not the reference builder's
    rt.close()


def test_autograd_refit_matches_gpu_builds(api, wl):
    import torch
    from illum_rt_gb300 import autograd
    sc = wl.icosphere(levels=4)
    rays = _dev(wl.camera_rays((0.0, 0.0, 3.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 50.0, 128, 128), np.float32)
    tris = sc.tris
    a, b = api.BatchRayTracer(0), api.BatchRayTracer(0)
    a.select("while-while")
    b.select("while-while")
    v = torch.from_numpy(sc.vpos[:, :3].copy()).cuda().requires_grad_(True)
    opt = torch.optim.SGD([v], lr=1e-3)
    for step in range(3):
        t1, b1, g1, r1 = autograd.closest_hits(a, v, tris, rays, builder="refit")
        t2, b2, g2, r2 = autograd.closest_hits(b, v, tris, rays, builder="gpu")
        h1 = torch.stack([t1, b1, g1, r1.view(torch.float32)], 1).detach().cpu().numpy()
        h2 = torch.stack([t2, b2, g2, r2.view(torch.float32)], 1).detach().cpu().numpy()
        assert_hits_match(h1, h2, False, f"refit step {step}")
        hit = t1 < 3e38
        loss = (t1[hit] * t1[hit]).sum() + b1[hit].sum()
        opt.zero_grad()
        loss.backward()
        assert torch.isfinite(v.grad).all() and v.grad.abs().sum() > 0
        opt.step()
    a.close()
    b.close()


def test_autograd_refit_rebuilds_for_new_topology(api, wl):
    """A triangle array with the same vertex count but other contents, whether a new array or
    the old one edited in place, gets a tree of its own: the refit builder never refits a tree
    built for other triangles."""
    import torch
    from illum_rt_gb300 import autograd
    sc = wl.icosphere(levels=4)
    rays = _dev(wl.camera_rays((0.0, 0.0, 3.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 50.0, 128, 128), np.float32)
    a, b = api.BatchRayTracer(0), api.BatchRayTracer(0)
    a.select("while-while")
    b.select("while-while")
    v = torch.from_numpy(sc.vpos[:, :3].copy()).cuda()
    perm = np.random.default_rng(11).permutation(sc.tris.shape[0])
    tris = sc.tris.copy()
    autograd.closest_hits(a, v, tris, rays, builder="refit")
    for kind in ("new array", "edited in place"):
        if kind == "new array":
            tris = np.ascontiguousarray(tris[perm])
        else:
            tris[:] = tris[np.roll(np.arange(tris.shape[0]), 7)]
            tris[:, :3] = tris[:, [0, 2, 1]]  # the same triangles wound the other way
        t1, b1, g1, r1 = autograd.closest_hits(a, v, tris, rays, builder="refit")
        t2, b2, g2, r2 = autograd.closest_hits(b, v, tris, rays, builder="gpu")
        h1 = torch.stack([t1, b1, g1, r1.view(torch.float32)], 1).cpu().numpy()
        h2 = torch.stack([t2, b2, g2, r2.view(torch.float32)], 1).cpu().numpy()
        assert same_bits(h1, h2).all(), kind
    a.close()
    b.close()
