"""On-disk cache of built trees (grt_set_bvh_cache): a second build of the same scene and
options is served from the cache with an identical tree and identical hits; other options or a
damaged file cost a build, never a wrong tree; scene sets use the cache per scene."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _needs_cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _hits(rt, rays_np):
    import torch
    rays = torch.from_numpy(rays_np).cuda()
    hits = torch.zeros((rays.shape[0], 4), device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    rt.trace(rays, hits, False, s)
    rt.check(s)
    return hits.cpu().numpy()


def test_cache_hit_gives_the_same_tree(api, wl, tmp_path):
    sc, rays = wl.heightfield_primary()
    rt = api.BatchRayTracer(0)
    rt.set_bvh_cache(str(tmp_path))
    rt.build(sc.vpos, sc.tris)
    assert rt.cache_stats() == (0, 1)
    first = rt.export_bvh()
    h1 = _hits(rt, rays)
    files = os.listdir(tmp_path)
    assert len(files) == 1 and files[0].startswith("grt-") and files[0].endswith(".bvh")
    rt.build(sc.vpos, sc.tris)
    assert rt.cache_stats() == (1, 1)
    second = rt.export_bvh()
    assert all(np.array_equal(a, b) for a, b in zip(first[:2], second[:2])) and first[2] == second[2]
    assert (h1.view(np.uint32) == _hits(rt, rays).view(np.uint32)).all()
    # other options: another file
    rt.build(sc.vpos, sc.tris, max_tris=2)
    assert rt.cache_stats() == (1, 2) and len(os.listdir(tmp_path)) == 2
    # a damaged file is rebuilt and rewritten, with the right tree
    path = tmp_path / files[0]
    data = bytearray(path.read_bytes())
    data[200:260] = b"\xff" * 60
    path.write_bytes(bytes(data))
    rt.build(sc.vpos, sc.tris)
    assert rt.cache_stats() == (1, 3)
    third = rt.export_bvh()
    assert all(np.array_equal(a, b) for a, b in zip(first[:2], third[:2]))
    rt.build(sc.vpos, sc.tris)
    assert rt.cache_stats() == (2, 3)
    # a header that announces more nodes than the file holds (its node count at byte 56) costs a
    # build, and nothing of the announced size is allocated
    data = bytearray(path.read_bytes())
    data[56:64] = (1 << 24).to_bytes(8, "little")
    path.write_bytes(bytes(data))
    rt.build(sc.vpos, sc.tris)
    assert rt.cache_stats() == (2, 4)
    assert all(np.array_equal(a, b) for a, b in zip(first[:2], rt.export_bvh()[:2]))
    # a changed vertex is another scene
    v = sc.vpos.copy()
    v[7, 2] += 0.01
    rt.build(v, sc.tris)
    assert rt.cache_stats() == (2, 5)
    rt.set_bvh_cache(None)
    rt.build(sc.vpos, sc.tris)
    assert rt.cache_stats() == (2, 5)
    with pytest.raises(api.GRTError):
        rt.set_bvh_cache(str(tmp_path / "does-not-exist"))
    rt.close()


def test_scene_sets_use_the_cache(api, wl, tmp_path):
    scenes = [(s.vpos, s.tris) for s in (wl.soup(61, 2000), wl.soup(62, 5000), wl.soup(63, 300))]
    rt = api.BatchRayTracer(0)
    rt.set_bvh_cache(str(tmp_path))
    rt.build_scenes(scenes)
    assert rt.cache_stats() == (0, 3)
    rt.build_scenes(scenes)
    assert rt.cache_stats() == (3, 3)
    rt.close()
