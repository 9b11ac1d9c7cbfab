"""Host logic of bench.py that the benchmark line depends on: the tuned tree options read from
the tuning table, and the figures read from the committed ncu summary of the fused kernel."""
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def test_tree_options_default_to_the_reference_cuda_build():
    assert bench.tree_options({}) == {"max_tris": 4, "planes": 16, "esc": True}
    assert bench.tree_label({}) == "SAH 16 planes, ESC, leaf<=4"


def test_tree_options_of_the_committed_spheres_entry():
    with open(os.path.join(ROOT, "illum-rt_gb300", "tuning.json")) as f:
        table = json.load(f)
    entry = table["NVIDIA GB300|spheres"]
    opts = bench.tree_options(entry)
    assert opts == {"max_tris": entry["max_tris"], "planes": entry["planes"], "esc": bool(entry["esc"])}
    assert bench.tree_label(entry) == "SAH %d planes, %s, leaf<=%d" % (
        entry["planes"], "ESC" if entry["esc"] else "no ESC", entry["max_tris"])


def test_load_tuning_falls_back_to_the_spheres_entry():
    spheres = bench.load_tuning("NVIDIA GB300", "spheres")
    assert bench.load_tuning("NVIDIA GB300", "no-such-scene") == spheres
    assert bench.load_tuning("no such GPU", "spheres") == bench.load_tuning("no such GPU", "soups64")


def test_profile_figures_are_present_and_plausible():
    traffic = bench.profile_figure("dram_bytes_per_launch")
    l2 = bench.profile_figure("l2_bytes_per_bounce_ray")
    assert traffic is not None and 1e6 < traffic < 1e10
    # L2 bytes per bounce ray: above a ray and its hit (48 B), below the algorithmic bytes of the
    # deepest plausible traversal
    assert l2 is not None and 48 < l2 < 10000
    assert bench.profile_figure("no_such_key") is None
