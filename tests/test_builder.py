"""The product's host builder (grt_host_bvh_*, the code grt_build runs) produces the
reference's BVH node for node: against the golden digests made by the reference itself, and
against the oracle on the full benchmark scenes."""
import numpy as np
import pytest

import cases
from conftest import GOLDEN_CASES, load_golden
from make_golden import bvh_digest


@pytest.mark.parametrize("name", GOLDEN_CASES)
@pytest.mark.parametrize("bname,opts", cases.BUILDERS, ids=[b for b, _ in cases.BUILDERS])
def test_builder_matches_reference_digest(api, golden_scenes, name, bname, opts):
    g = load_golden(name)
    v, t, _, _ = golden_scenes[name]
    nodes, index, root = api.HostBVH(v, t, **opts).export()
    assert nodes.shape[0] == int(g["nodes_" + bname])
    assert (bvh_digest(nodes, index, root) == g["bvh_" + bname]).all()


@pytest.mark.parametrize("scene", ["spheres", "icosphere", "soup"])
def test_builder_matches_oracle_full_scenes(api, orc, wl, scene):
    sc = {"spheres": wl.spheres, "icosphere": wl.icosphere, "soup": lambda: wl.soup(9, 150000)}[scene]()
    h = api.HostBVH(sc.vpos, sc.tris)
    nodes, index, root = h.export()
    o = orc.OracleBVH(sc.vpos, sc.tris)
    assert root == o.root
    assert np.array_equal(nodes, o.nodes()) and np.array_equal(index, o.index())
    assert h.stats["depth"] == o.depth()


def test_builder_rejects_bad_input(api):
    v = np.zeros((3, 4), np.float32)
    t = np.array([[0, 1, 5, 0]], np.uint32)  # vertex 5 does not exist
    with pytest.raises(api.GRTError):
        api.HostBVH(v, t)
    with pytest.raises(api.GRTError):
        api.HostBVH(v, np.array([[0, 1, 2, 0]], np.uint32), max_tris=0)


def test_builder_empty_and_tiny(api):
    v = np.array([[0, 0, 0, 1], [1, 0, 0, 1], [0, 1, 0, 1]], np.float32)
    nodes, index, root = api.HostBVH(v, np.zeros((0, 4), np.uint32), esc=False).export()
    assert nodes.shape[0] == 1 and index.size == 0 and nodes[0, 13] == 0  # one empty leaf
    nodes, index, root = api.HostBVH(v, np.array([[0, 1, 2, 0]], np.uint32)).export()
    assert nodes.shape[0] == 1 and list(index) == [0]
