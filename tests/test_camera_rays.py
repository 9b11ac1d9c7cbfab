"""Camera rays of the primary-ray step (grt_camera_rays), as the reference's cam_ray
(libgi/camera.cpp:11-28) computes them: the oracle's float restatement equals the reference's
own cam_ray on the golden cases (tests/golden/golden_camera.npz, written by
make_golden_camera.py from the reference build) and, where the reference build is present, live
at 1024x1024 (CPU). The GPU kernel is checked against both in test_raygen_gpu.py."""
import numpy as np
import pytest

from make_golden_camera import camera_cases

GOLDEN = None


def _golden():
    global GOLDEN
    if GOLDEN is None:
        import os
        GOLDEN = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "golden_camera.npz")))
    return GOLDEN


@pytest.mark.parametrize("case", camera_cases(), ids=lambda c: c[0])
def test_oracle_equals_reference_golden(orc, case):
    name, pos, d, up, nw, nh, w, h, mode, seed, _ = case
    g = _golden()
    off = g.get(name + "/offsets")
    got = orc.cam_rays(pos, d, up, nw, nh, w, h, off, mode == "jitter", seed)
    assert (got.view(np.uint32) == g[name + "/rays"].view(np.uint32)).all()


def test_oracle_equals_reference_live_full_size(orc):
    d = np.array((0.0, 0.0, -1.0), np.float32)
    want = orc.ref_cam_rays((0.0, 0.0, 35.0), d, (0.0, 1.0, 0.0), 0.6370703, 0.6370703, 1024, 1024, None, True, 99)
    if want is None:
        pytest.skip("reference build absent")
    got = orc.cam_rays((0.0, 0.0, 35.0), d, (0.0, 1.0, 0.0), 0.6370703, 0.6370703, 1024, 1024, None, True, 99)
    assert (got.view(np.uint32) == want.view(np.uint32)).all()
