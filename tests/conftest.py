"""Shared test setup: the `gpu` marker, package/oracle loading and golden fixtures."""
from __future__ import annotations

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (ROOT, GOLDEN):
    if p not in sys.path:
        sys.path.insert(0, p)

import __graft_entry__ as ge  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


@pytest.fixture(scope="session")
def pkg():
    ge.build()
    return ge.load_package()


@pytest.fixture(scope="session")
def orc(pkg):
    return ge.load_oracle()


@pytest.fixture(scope="session")
def wl(pkg):
    from illum_rt_gb300 import workloads
    return workloads


@pytest.fixture(scope="session")
def api(pkg):
    from illum_rt_gb300 import api as a
    return a


def load_golden(name: str):
    return dict(np.load(os.path.join(GOLDEN, f"golden_{name}.npz")))


@pytest.fixture(scope="session")
def gpu_tracer(api):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    rt = api.BatchRayTracer(0)
    yield rt
    rt.close()


def same_bits(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Per-row equality of float32 [n, 4] hit records as raw bits."""
    return (np.ascontiguousarray(a, np.float32).view(np.uint32) ==
            np.ascontiguousarray(b, np.float32).view(np.uint32)).all(axis=1)


GOLDEN_CASES = ["heightfield", "spheres", "kat", "soup3000", "icosphere3"]


@pytest.fixture(scope="session")
def golden_scenes(pkg):
    """name -> (vpos, tris, rays, any_rays) with the rays taken from the fixture where stored."""
    import make_golden
    out = {}
    for name, (v, t, rays, stored, _) in make_golden.scenes().items():
        g = load_golden(name)
        if stored:
            rays = g["rays"]
        out[name] = (v, t, rays, g["any_rays"])
    return out


NEAR_TIE = 1e-6  # |t1 - t2| <= NEAR_TIE * t: the documented near-tie class


def assert_hits_match(got: np.ndarray, want: np.ndarray, exact: bool, what: str = "hits"):
    """Exact tracers: every hit record bit-identical. Speculative tracers: rows may name a
    different triangle only as a near-tie (both hit, |t1 - t2| <= 1e-6 t); rows naming the same
    triangle are bit-identical."""
    g = np.ascontiguousarray(got, np.float32)
    w = np.ascontiguousarray(want, np.float32)
    same = same_bits(g, w)
    if exact:
        bad = ~same
        assert not bad.any(), f"{bad.sum()} of {bad.size} {what} differ, first rows {np.nonzero(bad)[0][:5]}"
        return 0
    diff_ref = g.view(np.uint32)[:, 3] != w.view(np.uint32)[:, 3]
    assert (same | diff_ref).all(), f"{what}: same triangle but different t/beta/gamma"
    rows = np.nonzero(diff_ref)[0]
    tg, tw = g[rows, 0].astype(np.float64), w[rows, 0].astype(np.float64)
    near = (tg < 3e38) & (tw < 3e38) & (np.abs(tg - tw) <= NEAR_TIE * np.abs(tw))
    assert near.all(), f"{what}: {(~near).sum()} differences are not near-ties, rows {rows[~near][:5]}"
    return int(rows.size)
