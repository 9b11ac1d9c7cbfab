"""Host logic of bench.py that the benchmark line depends on: the tuned tree options read from
the tuning table, the figures read from the committed ncu summary of the fused kernel, and the
timing loop of the CPU baseline."""
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


def test_limiter_figures_come_from_the_committed_capture():
    lim = bench.limiter_figures()
    assert lim is not None and lim["kind"]
    assert 1 <= lim["lanes_per_instruction"] <= 32
    assert 0 < lim["issue_active_pct"] <= 100 and 0 < lim["l2_throughput_pct"] <= 100


def _hits(n, seed):
    import numpy as np
    g = np.random.default_rng(seed)
    h = np.zeros((n, 4), np.float32)
    h[:, 0] = g.uniform(1, 50, n).astype(np.float32)
    h[:, 1:3] = g.uniform(0, 0.5, (n, 2)).astype(np.float32)
    h[:, 3] = g.integers(0, 1 << 20, n).astype(np.uint32).view(np.float32)
    return h


def test_classify_hits_near_ties_and_mismatches():
    import numpy as np
    want = _hits(1000, 1)
    got = want.copy()
    assert bench.classify_hits(got, want) == {"differing": 0, "all_near_ties": True, "not_near_ties": 0}
    # another triangle at a t within 1e-6 t: a near-tie
    got[5, 3] = np.uint32(7).view(np.float32)
    got[5, 0] = np.nextafter(want[5, 0], np.float32(1e9))
    r = bench.classify_hits(got, want)
    assert r["differing"] == 1 and r["all_near_ties"]
    # the same triangle with another beta: never a near-tie
    got[9, 1] += np.float32(0.01)
    r = bench.classify_hits(got, want)
    assert r["differing"] == 2 and not r["all_near_ties"] and r["not_near_ties"] == 1
    # another triangle far away, and a miss against a hit
    got = want.copy()
    got[3, 3] = np.uint32(8).view(np.float32)
    got[3, 0] = want[3, 0] * np.float32(1.01)
    got[4, 0] = np.float32(3.4028234663852886e38)
    got[4, 3] = np.uint32(9).view(np.float32)
    assert bench.classify_hits(got, want)["not_near_ties"] == 2


def test_classify_paths_first_differing_bounce():
    import numpy as np
    n, b = 200, 5
    bh_o = _hits(n * b, 2).reshape(n, b, 4)
    res_o = np.random.default_rng(3).integers(0, 1 << 30, (n, 4)).astype(np.uint32)
    res_g, bh_g = res_o.copy(), bh_o.copy()
    assert bench.classify_paths(res_g, bh_g, res_o, bh_o)["differing"] == 0
    # path 10 leaves through a near-tie at bounce 2 and then differs in everything after it
    bh_g[10, 2, 3] = np.uint32(12345).view(np.float32)
    bh_g[10, 2, 0] = np.nextafter(bh_o[10, 2, 0], np.float32(0))
    bh_g[10, 3:] = _hits(2, 9)
    res_g[10] += 1
    r = bench.classify_paths(res_g, bh_g, res_o, bh_o)
    assert r == {"differing": 1, "all_near_ties": True, "not_near_ties": 0}
    # path 20: results differ but every bounce hit agrees (a shading mismatch)
    res_g[20, 0] ^= 1
    r = bench.classify_paths(res_g, bh_g, res_o, bh_o)
    assert r["differing"] == 2 and r["not_near_ties"] == 1
    # path 30: first differing hit is far from the oracle's
    res_g[20] = res_o[20]
    bh_g[30, 0, 0] = bh_o[30, 0, 0] * np.float32(2)
    bh_g[30, 0, 3] = np.uint32(1).view(np.float32)
    r = bench.classify_paths(res_g, bh_g, res_o, bh_o)
    assert r["differing"] == 2 and r["not_near_ties"] == 1


def test_cpu_baseline_repeats_until_enough_work():
    """One untimed warm-up step, then steps until both the time and the repetition minimum are
    reached; the rate is the median of the repetitions."""

    class FakeStep:
        calls = 0

        def run(self):
            self.calls += 1
            return 1_000_000 * self.calls, 0.5

        def cores(self):
            return 7

    f = FakeStep()
    rate, reps, n, t, cores = bench.cpu_baseline(f, min_seconds=1.2, min_reps=2)
    assert f.calls == 4 and reps == 3 and t == 1.5 and cores == 7
    assert n == (2 + 3 + 4) * 1_000_000
    assert rate == 6.0  # median of 4, 6 and 8 Mrays/s
    f = FakeStep()
    rate, reps, n, t, cores = bench.cpu_baseline(f, min_seconds=0.1, min_reps=5)
    assert f.calls == 6 and reps == 5 and rate == 8.0  # median of 4, 6, 8, 10, 12
