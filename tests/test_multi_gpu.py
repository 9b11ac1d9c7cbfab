"""Many scenes with uneven ray batches in one launch (grt_build_scenes / grt_trace_multi): every
batch's hits equal the oracle's for its scene (bit-exact for the exact loop orders, near-ties
only for the speculative ones), the per-scene BVHs are the reference builder's, and empty
scenes and empty batches are handled."""
import numpy as np
import pytest

from conftest import assert_hits_match

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _needs_cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


@pytest.fixture(scope="module")
def multi_case(api, orc, wl):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    scenes, rays, oracles = [], [], []
    for i in range(12):
        ntri = wl.log_uniform(91, 2 * i, 1024, 1 << 16)
        nray = wl.log_uniform(91, 2 * i + 1, 4096, 1 << 16)
        sc = wl.soup(100 + i, ntri, sigma=0.5)
        lo, hi = sc.bounds()
        scenes.append((sc.vpos, sc.tris))
        rays.append(wl.shell_rays(200 + i, lo, hi, nray))
        oracles.append(orc.OracleBVH(sc.vpos, sc.tris))
    # an empty scene
    scenes.append((np.zeros((3, 4), np.float32), np.zeros((0, 4), np.uint32)))
    rays.append(rays[0][:100].copy())
    oracles.append(None)
    rt = api.BatchRayTracer(0)
    stats = rt.build_scenes(scenes, esc=True)
    d_rays = [torch.from_numpy(r).cuda() for r in rays]
    yield dict(rt=rt, scenes=scenes, rays=rays, d_rays=d_rays, oracles=oracles, stats=stats)
    rt.close()


def test_scene_bvhs_are_the_reference_builders(multi_case):
    rt = multi_case["rt"]
    for i, o in enumerate(multi_case["oracles"]):
        if o is None:
            continue
        st = multi_case["stats"][i]
        nodes, index, root = rt.export_scene_bvh(i, st["ref_nodes"], st["tri_records"])
        assert root == o.root and np.array_equal(nodes, o.nodes()) and np.array_equal(index, o.index())


@pytest.mark.parametrize("tracer", ["persistent-while-while", "persistent-if-if", "persistent-speculative-while-while",
                                    "persistent-bvh4-speculative-while-while"])
@pytest.mark.parametrize("any_hit", [False, True])
def test_multi_batches_match_oracle(multi_case, tracer, any_hit):
    import torch
    rt = multi_case["rt"]
    rt.select(tracer)
    # batches in a shuffled scene order, one scene twice, plus an empty batch
    order = [5, 0, 12, 3, 11, 7, 1, 9, 2, 10, 4, 8, 6, 3]
    batches, outs, src = [], [], []
    for s in order:
        r = multi_case["d_rays"][s]
        if any_hit:
            r = r.clone()
            r[:, 7] = 1.5  # finite t_max so that occlusion is not trivial
        h = torch.zeros((r.shape[0], 4), device="cuda")
        batches.append((s, r, h))
        outs.append(h)
        src.append(r)
    batches.append((0, multi_case["d_rays"][0][:0], torch.zeros((0, 4), device="cuda")))
    stream = torch.cuda.current_stream().cuda_stream
    rt.trace_multi(batches, any_hit=any_hit, stream=stream)
    rt.check(stream, timeout_ms=60000)
    for s, h, r in zip(order, outs, src):
        got = h.cpu().numpy()
        o = multi_case["oracles"][s]
        rays = r.cpu().numpy()
        if o is None:  # empty scene: all miss
            assert (got[:, 0] == np.float32(3.4028234663852886e38)).all()
            continue
        if any_hit:
            occ = (got.view(np.uint32)[:, 3] == 0xFFFFFFFF).astype(np.uint8)
            assert (occ == o.any(rays)[0]).all(), (tracer, s)
        else:
            assert_hits_match(got, o.closest(rays)[0], "speculative" not in tracer, f"{tracer} scene {s}")
    rt.select("while-while")
