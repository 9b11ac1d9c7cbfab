"""The oracle's own copy of the benchmark workload (oracle/scenes.cpp), which the benchmark's
CPU legs use so that they load only the oracle, equals the library's workload generators bit for
bit: the sphere scene, its 1024x1024 primary rays, and camera rays of other shapes."""
import hashlib

import numpy as np
import pytest


def _digest(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def test_spheres_workload_equals_library_generator(orc, wl):
    sc, rays = wl.spheres_primary(res=1024)
    v, t, r = orc.spheres_primary(res=1024)
    assert _digest(v, t) == _digest(sc.vpos, sc.tris)
    assert _digest(r) == _digest(rays)


@pytest.mark.parametrize("count,slices,stacks", [(3, 16, 8), (5, 32, 16), (2, 8, 4)])
def test_sphere_shapes(orc, wl, count, slices, stacks):
    sc = wl.spheres(seed=9, count=count, slices=slices, stacks=stacks)
    v, t = orc.spheres_scene(seed=9, count=count, slices=slices, stacks=stacks)
    assert (v.view(np.uint32) == sc.vpos.view(np.uint32)).all()
    assert (t == sc.tris).all()


@pytest.mark.parametrize("pos,look,fovy,w,h", [((0.5, -1.0, 1.0), (0.5, 0.5, 0.0), 65.0, 256, 256),
                                                ((0.0, 0.0, 3.0), (0.0, 0.0, 0.0), 50.0, 128, 96),
                                                ((1.0, 2.0, 3.0), (-2.0, 0.5, 0.0), 120.0, 64, 200)])
def test_camera_rays(orc, wl, pos, look, fovy, w, h):
    want = wl.camera_rays(pos, look, (0.0, 1.0, 0.0), fovy, w, h)
    got = orc.camera_rays(pos, look, (0.0, 1.0, 0.0), fovy, w, h)
    assert (got.view(np.uint32) == want.view(np.uint32)).all()
