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
