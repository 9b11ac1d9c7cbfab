"""The reference tracer's `bvh export <depth> <file.obj>` and `bvh statistics` commands
(rt/cpu/bvh2.cpp:228-317) on the product builder's trees: the exported OBJ text and the printed
statistics equal the reference's (golden_bvh_tools.npz, and live where oracle/_ref exists)."""
import numpy as np
import pytest

import cases
from conftest import GOLDEN_CASES, load_golden
from make_golden import TOOL_DEPTHS, array_digest


def _stats_text(st):
    return (f"number of leaf nodes: {st['leaves']}\nminimum triangles per node: {st['min_tris']}\n"
            f"maximum triangles per node: {st['max_tris']}\naverage triangles per node: {st['avg_tris']}\n"
            f"median of triangles per node: {st['median_tris']}\n")


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_export_and_statistics_match_reference(api, golden_scenes, name, tmp_path):
    v, t, _, _ = golden_scenes[name]
    g = load_golden("bvh_tools")
    h = api.HostBVH(v, t, **dict(cases.BUILDERS[0][1]))
    for d in TOOL_DEPTHS:
        path = tmp_path / f"{name}_{d}.obj"
        h.export_obj(d, path)
        assert (array_digest(np.frombuffer(path.read_bytes(), np.uint8)) == g[f"obj_{name}_{d}"]).all(), (name, d)
    assert _stats_text(h.leaf_stats()) == bytes(g[f"stats_{name}"]).decode()


@pytest.mark.parametrize("seed,ntri", [(41, 37), (42, 1000), (43, 20000)])
def test_export_and_statistics_live(api, orc, wl, seed, ntri, tmp_path):
    if not orc.ref_available():
        pytest.skip("reference build (oracle/_ref) not present on this host")
    sc = wl.soup(seed, ntri, sigma=0.5)
    opts = dict(split="sah", max_tris=3, planes=8, esc=True)
    h = api.HostBVH(sc.vpos, sc.tris, **opts)
    ref = orc.ReferenceBVH(sc.vpos, sc.tris, **opts)
    for d in (2, 7, 40):
        ours, theirs = tmp_path / "ours.obj", tmp_path / "ref.obj"
        h.export_obj(d, ours)
        orc.ref_bvh_command(ref, f"export {d} {theirs}")
        assert ours.read_bytes() == theirs.read_bytes(), d
    assert _stats_text(h.leaf_stats()) == orc.ref_bvh_command(ref, "statistics")


def test_statistics_quirks(api):
    """The first leaf only sets the minimum (the reference's else-if), so a tree of one leaf
    reports a maximum of 0; two leaves have no median in the reference (it reads past the end),
    so that is an error here."""
    v = np.zeros((6, 4), np.float32)
    v[:, 0] = [0.0, 1.0, 0.0, 10.0, 11.0, 10.0]
    v[:, 1] = [0.0, 0.0, 1.0, 0.0, 0.0, 1.0]
    one_leaf = np.array([[0, 1, 2, 0]] * 3, np.uint32)  # three coincident triangles
    st = api.HostBVH(v, one_leaf, split="sah", max_tris=4, planes=16, esc=False).leaf_stats()
    assert (st["leaves"], st["min_tris"], st["max_tris"], st["avg_tris"], st["median_tris"]) == (1, 3, 0, 3, 3)
    two_leaves = np.array([[0, 1, 2, 0], [3, 4, 5, 0]], np.uint32)
    with pytest.raises(api.GRTError):
        api.HostBVH(v, two_leaves, split="sah", max_tris=1, planes=16, esc=False).leaf_stats()


def test_interprete_knows_the_cpu_tracer_commands(api):
    rt = api.BatchRayTracer.__new__(api.BatchRayTracer)  # no device needed for the settings
    rt.bvh_type, rt.bvh_max_tris_per_node, rt.bvh_planes = "sah", 4, 16
    assert rt.interprete("bvh om") and rt.bvh_type == "om"
    assert rt.interprete("bvh sah 8") and (rt.bvh_type, rt.bvh_planes) == ("sah", 8)
    assert rt.interprete("bvh triangles multiple 6") and rt.bvh_max_tris_per_node == 6
    assert rt.interprete("bvh triangles single") and rt.bvh_max_tris_per_node == 1
    assert not rt.interprete("bvh frobnicate")
