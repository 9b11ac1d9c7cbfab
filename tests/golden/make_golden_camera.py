"""Generates golden_camera.npz from the REFERENCE's own cam_ray (libgi/camera.cpp:11-28).

Needs oracle/_ref/libref_sampling.so, which oracle/build_ref.sh compiles from the unmodified
reference source libgi/camera.cpp and the reference's sampling headers. Each case is a camera
(position, normalised view direction, up, near_w, near_h), an image size and an offset mode
(pixel centres, the PCG32 jitter of grt_camera_rays with a seed, or explicit offsets stored in
the fixture); the fixture holds the reference's rays in the grt_trace layout.

Run from the repository root:  python tests/golden/make_golden_camera.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

import __graft_entry__ as ge  # noqa: E402


def camera_cases():
    """(name, pos, dir, up, near_w, near_h, w, h, mode, seed, offsets or None)."""
    out = []
    specs = [("heightfield", (0.5, -1.0, 1.0), (0.0, 1.5, -1.0), (0.0, 1.0, 0.0), 0.6370703, 0.6370703, 64, 48),
             ("spheres", (0.0, 0.0, 35.0), (0.0, 0.0, -1.0), (0.0, 1.0, 0.0), 0.6370703, 0.6370703, 80, 80),
             ("oblique", (1.0, 2.0, 3.0), (-0.6, -0.3, -0.74), (0.0, 1.0, 0.0), 1.2, 0.9, 33, 17)]
    for name, pos, d, up, nw, nh, w, h in specs:
        d = np.asarray(d, np.float64)
        d = tuple(float(x) for x in (d / np.linalg.norm(d)).astype(np.float32))
        out.append((name + "_centre", pos, d, up, nw, nh, w, h, "centre", 0, None))
        out.append((name + "_jitter", pos, d, up, nw, nh, w, h, "jitter", 17, None))
        off = (np.random.default_rng(len(out)).random((w * h, 2)) - 0.5).astype(np.float32)
        out.append((name + "_offsets", pos, d, up, nw, nh, w, h, "offsets", 0, off))
    return out


def main():
    ge.build()
    orc = ge.load_oracle()
    store = {}
    for name, pos, d, up, nw, nh, w, h, mode, seed, off in camera_cases():
        rays = orc.ref_cam_rays(pos, d, up, nw, nh, w, h, off, mode == "jitter", seed)
        if rays is None:
            raise SystemExit("oracle/_ref/libref_sampling.so is missing: build it from the reference sources")
        store[name + "/rays"] = rays
        if off is not None:
            store[name + "/offsets"] = off
    np.savez_compressed(os.path.join(HERE, "golden_camera.npz"), **store)
    print("wrote golden_camera.npz with", len(camera_cases()), "cases")


if __name__ == "__main__":
    main()
