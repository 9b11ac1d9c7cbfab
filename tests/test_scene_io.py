"""OBJ / MTL scenes (scene_io.load_obj) in the library's layouts, with the reference importer's
material rules; a host BVH export (the reference's `bvh export` OBJ) reads back as geometry."""
import math

import numpy as np
import pytest


@pytest.fixture(scope="module")
def scene_io(pkg):
    from illum_rt_gb300 import scene_io
    return scene_io


def test_geometry_faces_and_materials(scene_io, tmp_path):
    (tmp_path / "m.mtl").write_text(
        "newmtl red\nKd 0.5 0.1 0.1\nNs 98\nNi 1.0\n"
        "newmtl lamp\nKd 0 0 0\nKs 0.25 0.25 0.25\nKe 4 4 3\nNi 1.5\n")
    (tmp_path / "s.obj").write_text(
        "# a quad, a triangle and a pentagon\nmtllib m.mtl\n"
        "v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nv 2 0 0\nv 3 0 0\nv 3 1 0\nv 2.5 2 0\nv 2 1 0\n"
        "vt 0 0\nvn 0 0 1\n"
        "f 1 2 3\n"
        "usemtl red\nf 1/1/1 2/1/1 3/1/1 4/1/1\n"
        "usemtl lamp\nf -5 -4 -3 -2 -1\n"
        "usemtl unknown\nf 1//1 3//1 4//1\n")
    v, t, names, mats = scene_io.load_obj(str(tmp_path / "s.obj"))
    assert v.shape == (9, 4) and v.dtype == np.float32 and (v[:, 3] == 1).all()
    assert names == ["", "red", "lamp", "unknown"]
    want = [(0, 1, 2, 0), (0, 1, 2, 1), (0, 2, 3, 1), (4, 5, 6, 2), (4, 6, 7, 2), (4, 7, 8, 2), (0, 2, 3, 3)]
    assert t.dtype == np.uint32 and [tuple(r) for r in t.tolist()] == want
    assert mats.shape == (4, 8)
    assert mats[0].tolist() == pytest.approx([0, 0, 0, 0, 0, 0, 1.3, 0.1])  # no material: the default
    red = mats[1]
    assert red[0] == pytest.approx(0.5 ** 2.2, rel=1e-6) and red[1] == pytest.approx(0.1 ** 2.2, rel=1e-5)
    assert red[6] == pytest.approx(1.3) and red[7] == pytest.approx(math.sqrt(2 / 100), rel=1e-6)
    lamp = mats[2]
    assert lamp[0:3] == pytest.approx([0.25 ** 2.2] * 3, rel=1e-6)  # Kd is black: Ks is the albedo
    assert lamp[3:6].tolist() == [4, 4, 3] and lamp[6] == pytest.approx(1.5) and lamp[7] == pytest.approx(0.1)
    assert mats[3].tolist() == pytest.approx([0, 0, 0, 0, 0, 0, 1.3, 0.1])  # not in the library


def test_bad_index_and_short_face(scene_io, tmp_path):
    (tmp_path / "a.obj").write_text("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 4\n")
    with pytest.raises(ValueError):
        scene_io.load_obj(str(tmp_path / "a.obj"))
    (tmp_path / "b.obj").write_text("v 0 0 0\nv 1 0 0\nf 1 2\n")
    with pytest.raises(ValueError):
        scene_io.load_obj(str(tmp_path / "b.obj"))


def test_bvh_export_reads_back(scene_io, api, wl, tmp_path):
    sc = wl.heightfield()
    h = api.HostBVH(sc.vpos, sc.tris)
    path = tmp_path / "boxes.obj"
    h.export_obj(2, str(path))
    v, t, names, mats = scene_io.load_obj(str(path))
    assert v.shape[0] > 0 and t.shape[0] > 0 and (t[:, :3] < v.shape[0]).all()
    lo, hi = sc.bounds()
    assert (v[:, :3].min(0) >= lo - 1e-6).all() and (v[:, :3].max(0) <= hi + 1e-6).all()
