"""Host logic of the autotuner (CPU, no kernels): the speculative grid sweep visits every point,
keeps the fastest configuration, leaves that configuration set on the tracer, and the tuning
table keeps the other entries when one is written."""
import itertools
import json

import pytest


class FakeTracer:
    """Records set_tuning calls; the fake timer reads the last one."""

    def __init__(self):
        self.calls = []

    def set_tuning(self, **kw):
        self.calls.append(dict(kw))

    @property
    def current(self):
        return self.calls[-1]


BASE = {"tracer": "persistent-speculative-while-while", "max_tris": 2, "planes": 256, "esc": 0,
        "block_threads": 64, "refill_threshold": 28, "refill_period": 2, "ms": 2.5}


def _autotune(pkg):
    from illum_rt_gb300 import autotune
    return autotune


@pytest.mark.parametrize("quick", [False, True])
def test_spec_sweep_times_every_point_and_keeps_the_fastest(pkg, quick):
    at = _autotune(pkg)
    grid = at.SPEC_GRID_QUICK if quick else at.SPEC_GRID
    rt = FakeTracer()
    target = {k: v[-1] for k, v in grid.items()}  # the fastest point: the last value of every axis

    def timer():
        cur = rt.current
        # launch parameters stay those of the best launch at every point
        assert {k: cur[k] for k in ("block_threads", "refill_threshold", "refill_period")} == \
            {k: BASE[k] for k in ("block_threads", "refill_threshold", "refill_period")}
        return 1.0 + sum(abs(cur[k] - target[k]) for k in grid)

    lines = []
    out = at.spec_sweep(rt, dict(BASE), quick, lines.append, timer)
    n = 1
    for v in grid.values():
        n *= len(v)
    assert out.pop("_searched") == n == len(lines)
    seen = {tuple(json.loads(l)[k] for k in grid) for l in lines}
    assert seen == set(itertools.product(*grid.values()))
    assert out["ms"] == 1.0 and {k: out[k] for k in grid} == target
    assert {k: out[k] for k in BASE if k != "ms"} == {k: BASE[k] for k in BASE if k != "ms"}
    # the tracer is left at the chosen point
    assert {k: rt.current[k] for k in grid} == target


def test_spec_sweep_keeps_the_base_when_no_point_is_faster(pkg):
    at = _autotune(pkg)
    rt = FakeTracer()
    out = at.spec_sweep(rt, dict(BASE), True, lambda line: None, lambda: BASE["ms"] + 1.0)
    out.pop("_searched")
    assert out == BASE
    # every speculative parameter goes back to 0, the library's compiled default
    assert {k: rt.current[k] for k in at.SPEC_GRID} == {k: 0 for k in at.SPEC_GRID}


def test_spec_grid_keys_are_tuning_fields(pkg):
    at = _autotune(pkg)
    from illum_rt_gb300 import api
    assert set(at.SPEC_GRID) <= set(api.TUNING_KEYS)
    assert set(at.SPEC_GRID_QUICK) == set(at.SPEC_GRID)
    for k, v in at.SPEC_GRID_QUICK.items():
        assert set(v) <= set(at.SPEC_GRID[k])


def test_save_merges_into_the_table(pkg, tmp_path, monkeypatch):
    at = _autotune(pkg)
    table = tmp_path / "tuning.json"
    table.write_text(json.dumps({"GPU A|spheres": {"ms": 1.0}, "GPU B|spheres": {"ms": 2.0}}))
    monkeypatch.setattr(at, "TABLE", str(table))
    at.save({"ms": 3.0}, "GPU A", "soups64")
    at.save({"ms": 0.5}, "GPU B")
    got = json.loads(table.read_text())
    assert got == {"GPU A|spheres": {"ms": 1.0}, "GPU A|soups64": {"ms": 3.0}, "GPU B|spheres": {"ms": 0.5}}


def test_save_creates_the_table(pkg, tmp_path, monkeypatch):
    at = _autotune(pkg)
    table = tmp_path / "new.json"
    monkeypatch.setattr(at, "TABLE", str(table))
    at.save({"ms": 1.5, "tracer": "persistent-while-while"}, "GPU C")
    assert json.loads(table.read_text()) == {"GPU C|spheres": {"ms": 1.5, "tracer": "persistent-while-while"}}


def test_committed_entries_name_only_known_fields(pkg):
    at = _autotune(pkg)
    from illum_rt_gb300 import api
    with open(at.TABLE) as f:
        table = json.load(f)
    assert table, "the committed tuning table is empty"
    meta = {"ms", "searched", "seconds", "tracer", "max_tris", "planes", "esc"}
    for key, entry in table.items():
        gpu, scene = key.split("|")
        assert gpu and scene in ("spheres", "soups64")
        assert set(entry) <= set(api.TUNING_KEYS) | meta, key
        assert entry["tracer"] in api.TRACERS, key
