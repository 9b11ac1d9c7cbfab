"""GPU parity of the ray-generation steps and of the diffuse path tracer.

Every bounce ray is derived with correctly rounded IEEE operations only, so the GPU and the
oracle produce the same rays, hence the same hits, bit for bit, through all bounces. The
wavefront form, the fused persistent form and their CUDA-graph replays must agree with the
oracle and with each other on every path."""
import numpy as np
import pytest

from conftest import same_bits

pytestmark = pytest.mark.gpu

LIGHT = (0.0, 15.0, 0.0)


@pytest.fixture(autouse=True)
def _needs_cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


@pytest.fixture(scope="module")
def spheres_setup(api, orc, wl):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    sc, rays = wl.spheres_primary(res=512)
    o = orc.OracleBVH(sc.vpos, sc.tris)
    rt = api.BatchRayTracer(0)
    rt.build(sc.vpos, sc.tris)
    albedo = 0.3 + 0.6 * (np.arange(256) % 7) / 6.0
    rt.set_materials(albedo)
    d_rays = torch.from_numpy(rays).cuda()
    d_hits = torch.zeros((rays.shape[0], 4), device="cuda")
    rt.trace(d_rays, d_hits)
    rt.check()
    want, _ = o.closest(rays)
    assert same_bits(d_hits.cpu().numpy(), want).all()
    yield dict(sc=sc, rays=rays, o=o, rt=rt, d_rays=d_rays, d_hits=d_hits, prim_hits=want, albedo=albedo)
    rt.close()


def test_compact_hits_is_stable(spheres_setup):
    import torch
    s = spheres_setup
    n = s["rays"].shape[0]
    idx = torch.zeros(n, dtype=torch.int32, device="cuda")
    cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
    s["rt"].compact_hits(s["d_hits"], idx, cnt)
    torch.cuda.synchronize()
    want = np.nonzero(s["prim_hits"][:, 0] < np.float32(3.4028234663852886e38))[0]
    c = int(cnt.item())
    assert c == want.size
    assert (idx[:c].cpu().numpy() == want).all()


def test_shadow_rays_and_any_hit(spheres_setup):
    import torch
    s = spheres_setup
    n = s["rays"].shape[0]
    out = torch.zeros((n, 8), device="cuda")
    cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
    s["rt"].shadow_rays(s["d_rays"], s["d_hits"], LIGHT, 1e-4, out, cnt)
    torch.cuda.synchronize()
    want = s["o"].shadow_rays(s["rays"], s["prim_hits"], LIGHT, 1e-4)
    c = int(cnt.item())
    assert c == want.shape[0] > 0
    got = out[:c].cpu().numpy()
    assert (got.view(np.uint32) == want.view(np.uint32)).all()
    for tracer in ("while-while", "persistent-while-while"):
        s["rt"].select(tracer)
        hits = torch.zeros((c, 4), device="cuda")
        s["rt"].trace(out[:c], hits, any_hit=True)
        s["rt"].check()
        occ = (hits.cpu().numpy().view(np.uint32)[:, 3] == 0xFFFFFFFF).astype(np.uint8)
        assert (occ == s["o"].any(want)[0]).all()
    s["rt"].select("while-while")


@pytest.mark.parametrize("tracer", ["while-while", "if-if", "speculative-while-while", "bvh4-speculative-while-while"])
@pytest.mark.parametrize("mode,graph", [(0, 0), (1, 0), (0, 1), (1, 1)], ids=["wavefront", "fused", "wavefront-graph",
                                                                          "fused-graph"])
def test_pathtrace_matches_oracle(api, spheres_setup, mode, graph, tracer):
    import torch
    s = spheres_setup
    s["rt"].select(tracer)  # the loop order of the per-bounce and the fused kernels
    n_paths = 300_000
    params = api.BatchRayTracer.pt_params(mode=mode, use_graph=graph, seed=7)
    res = torch.zeros((n_paths, 4), dtype=torch.int32, device="cuda")
    bh = torch.zeros((n_paths, 5, 4), dtype=torch.float32, device="cuda")
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        for _ in range(2 if graph else 1):  # the second call replays the captured graph
            res.zero_()
            s["rt"].pathtrace(params, s["d_rays"], s["d_hits"], n_paths, res, bh, stream.cuda_stream)
        s["rt"].check(stream.cuda_stream)
    torch.cuda.synchronize()
    want, want_bh = s["o"].pathtrace(s["rays"], s["prim_hits"], n_paths, seed=7, albedo=s["albedo"], bounce_hits=True)
    got = res.cpu().numpy().view(np.uint32)
    got_bh = bh.cpu().numpy()
    bad = (got != want).any(axis=1)
    if "speculative" in tracer:
        # a path may leave the reference's only through a near-tie at its first differing bounce
        assert bad.sum() <= 1e-4 * n_paths
        for p in np.nonzero(bad)[0]:
            k = int(np.nonzero((got_bh[p].view(np.uint32) != want_bh[p].view(np.uint32)).any(axis=1))[0][0])
            tg, tw = float(got_bh[p, k, 0]), float(want_bh[p, k, 0])
            assert tg < 3e38 and tw < 3e38 and abs(tg - tw) <= 1e-6 * tw, (p, k, tg, tw)
        got, want_bh_cmp = got[~bad], want_bh[~bad]
        assert (got_bh[~bad].view(np.uint32) == want_bh_cmp.view(np.uint32)).all()
        got = res.cpu().numpy().view(np.uint32)
    else:
        assert not bad.any(), f"{bad.sum()} paths differ, first {np.nonzero(bad)[0][:5]}"
        assert (got_bh.view(np.uint32) == want_bh.view(np.uint32)).all()
    bounces = got[:, 1]
    assert bounces.min() >= 1 and bounces.max() == 5
    # Russian roulette before bounce ray 3: about 0.8 of the paths whose second bounce hit go on
    second_hit = (bounces >= 2) & (want_bh[:, 1, 0] < np.float32(3.4028234663852886e38))
    assert 0.75 < (bounces >= 3).sum() / max(1, second_hit.sum()) < 0.85
    s["rt"].select("while-while")


def test_pathtrace_no_primary_hit(api, spheres_setup):
    import torch
    s = spheres_setup
    hits = torch.zeros((16, 4), device="cuda")
    hits[:, 0] = float(np.float32(3.4028234663852886e38))
    res = torch.zeros((100, 4), dtype=torch.int32, device="cuda")
    for mode in (0, 1):
        s["rt"].pathtrace(api.BatchRayTracer.pt_params(mode=mode), s["d_rays"][:16], hits, 100, res)
        s["rt"].check()
        got = res.cpu().numpy().view(np.uint32)
        assert (got[:, 1] == 0).all() and (got[:, 2] == 0xFFFFFFFF).all()


def test_traversal_counts_equal_oracle(api, spheres_setup):
    """The counting kernel sees the oracle's visit sequence: equal inner-node and triangle-test
    totals over all bounce rays of the wavefront form."""
    import torch
    s = spheres_setup
    n_paths = 100_000
    cnt = torch.zeros(3, dtype=torch.int64, device="cuda")
    res = torch.zeros((n_paths, 4), dtype=torch.int32, device="cuda")
    s["rt"].set_traversal_counters(cnt)
    try:
        s["rt"].pathtrace(api.BatchRayTracer.pt_params(mode=0, seed=3), s["d_rays"], s["d_hits"], n_paths, res)
        s["rt"].check()
    finally:
        s["rt"].set_traversal_counters(None)
    totals = np.zeros(3, np.uint64)
    want, _ = s["o"].pathtrace(s["rays"], s["prim_hits"], n_paths, seed=3, albedo=s["albedo"], totals=totals)
    assert (res.cpu().numpy().view(np.uint32) == want).all()
    assert [int(x) for x in cnt.cpu().numpy()] == [int(x) for x in totals]
    assert int(totals[0]) == int(want[:, 1].sum())
