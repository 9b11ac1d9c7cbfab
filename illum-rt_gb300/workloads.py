"""Seeded synthetic workloads for the traversal benchmark and the parity tests.

The reference ships no scene files (its scripts load render-data/ models that are not
available), so each workload is generated from a seed by ``csrc/workloads.cpp`` through ctypes.
The generators use only IEEE basic operations and their own PCG32 stream, so the arrays are
bit-identical on every host. Layouts follow the reference's CUDA buffers:

* vertex positions ``float32[nv, 4]`` = (x, y, z, 1)            (rt/cuda/base.cpp:57-66)
* triangles        ``uint32[nt, 4]``  = (a, b, c, material)       (rt/cuda/base.cpp:49-53)
* rays             ``float32[n, 8]``  = (o.xyz, t_min, d.xyz, t_max) (rt/cuda/kernels.cu:52-60)

Scene definitions (sizes from the benchmark configurations):

* ``heightfield``: 64x64 vertex grid over [0,1]^2, heights U[0,0.2], 7,938 triangles; pinhole
  camera at (0.5,-1,1) looking at (0.5,0.5,0), up (0,1,0), fovy 65 deg, 256x256 pixel-centre rays.
* ``spheres``: 256 UV spheres of 32x16 quads (1,024 triangles each, 262,144 total) with centres
  U[-10,10]^3 and radii U[0.2,1.5]; camera at (0,0,35) looking at the origin, 1024x1024 rays.
* ``soup``: random triangle soups for the uneven multi-scene batch.
* ``icosphere``: icosahedron subdivided 6 times (81,920 triangles), radial displacement 0.05 N(0,1).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _libs

FLT_MAX = np.float32(3.4028234663852886e38)
RAY_EPS = np.float32(1e-4)  # ray::eps, libgi/rt.h:25


def _lib():
    return _libs.workloads()


def _fp(a):
    return a.ctypes.data_as(ctypes.c_void_p)


@dataclass
class Scene:
    name: str
    vpos: np.ndarray  # float32 [nv, 4]
    tris: np.ndarray  # uint32 [nt, 4]

    @property
    def nv(self) -> int:
        return int(self.vpos.shape[0])

    @property
    def nt(self) -> int:
        return int(self.tris.shape[0])

    def bounds(self):
        p = self.vpos[:, :3]
        return p.min(axis=0), p.max(axis=0)


def heightfield(seed: int = 1, n: int = 64, zmax: float = 0.2) -> Scene:
    v = np.zeros((n * n, 4), np.float32)
    t = np.zeros((2 * (n - 1) * (n - 1), 4), np.uint32)
    _lib().wl_heightfield(ctypes.c_uint64(seed), ctypes.c_uint32(n), ctypes.c_float(zmax), _fp(v), _fp(t))
    return Scene("heightfield", v, t)


def spheres(seed: int = 2, count: int = 256, slices: int = 32, stacks: int = 16, cext: float = 10.0,
            rmin: float = 0.2, rmax: float = 1.5) -> Scene:
    v = np.zeros((count * (stacks + 1) * slices, 4), np.float32)
    t = np.zeros((count * 2 * slices * stacks, 4), np.uint32)
    _lib().wl_spheres(ctypes.c_uint64(seed), ctypes.c_uint32(count), ctypes.c_uint32(slices),
                      ctypes.c_uint32(stacks), ctypes.c_float(cext), ctypes.c_float(rmin),
                      ctypes.c_float(rmax), _fp(v), _fp(t))
    return Scene("spheres", v, t)


def soup(seed: int, ntri: int, sigma: float = 0.5) -> Scene:
    v = np.zeros((3 * ntri, 4), np.float32)
    t = np.zeros((ntri, 4), np.uint32)
    _lib().wl_soup(ctypes.c_uint64(seed), ctypes.c_uint32(ntri), ctypes.c_float(sigma), _fp(v), _fp(t))
    return Scene("soup", v, t)


def icosphere(seed: int = 5, levels: int = 6, disp: float = 0.05) -> Scene:
    nv = 10 * 4 ** levels + 2
    nt = 20 * 4 ** levels
    v = np.zeros((nv, 4), np.float32)
    t = np.zeros((nt, 4), np.uint32)
    _lib().wl_icosphere(ctypes.c_uint64(seed), ctypes.c_uint32(levels), ctypes.c_float(disp), _fp(v), _fp(t))
    return Scene("icosphere", v, t)


def camera_rays(pos, look, up, fovy_deg: float, w: int, h: int, tmin: float = float(RAY_EPS)) -> np.ndarray:
    r = np.zeros((w * h, 8), np.float32)
    p = np.asarray(pos, np.float32)
    lk = np.asarray(look, np.float32)
    u = np.asarray(up, np.float32)
    _lib().wl_camera_rays(_fp(p), _fp(lk), _fp(u), ctypes.c_float(fovy_deg), ctypes.c_uint32(w),
                          ctypes.c_uint32(h), ctypes.c_float(tmin), _fp(r))
    return r


def shell_rays(seed: int, lo, hi, n: int, tmin: float = float(RAY_EPS)) -> np.ndarray:
    r = np.zeros((n, 8), np.float32)
    lo = np.ascontiguousarray(lo, np.float32)
    hi = np.ascontiguousarray(hi, np.float32)
    _lib().wl_sphere_shell_rays(ctypes.c_uint64(seed), _fp(lo), _fp(hi), ctypes.c_uint64(n),
                                ctypes.c_float(tmin), _fp(r))
    return r


def log_uniform(seed: int, seq: int, lo: int, hi: int) -> int:
    return int(_lib().wl_log_uniform(ctypes.c_uint64(seed), ctypes.c_uint64(seq), ctypes.c_uint64(lo),
                                     ctypes.c_uint64(hi)))


def normals(seed: int, n: int) -> np.ndarray:
    out = np.zeros(n, np.float32)
    _lib().wl_normals(ctypes.c_uint64(seed), ctypes.c_uint64(n), _fp(out))
    return out


# ---- the benchmark configurations -------------------------------------------------------

def heightfield_primary(res: int = 256):
    """Heightfield scene plus its 256x256 primary rays (the CPU-runnable configuration)."""
    sc = heightfield()
    rays = camera_rays((0.5, -1.0, 1.0), (0.5, 0.5, 0.0), (0.0, 1.0, 0.0), 65.0, res, res)
    return sc, rays


def spheres_primary(res: int = 1024):
    """Sphere scene (262,144 triangles) plus res x res coherent primary rays."""
    sc = spheres()
    rays = camera_rays((0.0, 0.0, 35.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 65.0, res, res)
    return sc, rays


def lit_spheres(count: int = 256, res: int = 1024):
    """Direct-lighting scene: `count` UV spheres (materials 0-3 by sphere), a floor at y = -12
    (material 4) and two emissive quads at y = 14 facing down (material 5), with its material
    table float32 [6, 8] (albedo rgb, emission rgb, ior, roughness) and res x res camera rays."""
    sc = spheres(count=count)
    per_sphere = 2 * 32 * 16
    tris = sc.tris.copy()
    tris[:, 3] = (np.arange(tris.shape[0]) // per_sphere) % 4
    quads = [((-30.0, -12.0, -30.0), (60.0, 60.0), 4, True),   # floor, normal up
             ((-6.0, 14.0, -3.0), (5.0, 6.0), 5, False),      # lights, normal down
             ((2.0, 14.0, -4.0), (5.0, 5.0), 5, False)]
    v = [sc.vpos]
    t = [tris]
    base = sc.vpos.shape[0]
    for (x0, y, z0), (dx, dz), mat, up in quads:
        q = np.array([[x0, y, z0, 1], [x0 + dx, y, z0, 1], [x0 + dx, y, z0 + dz, 1], [x0, y, z0 + dz, 1]], np.float32)
        v.append(q)
        tri = [(0, 2, 1), (0, 3, 2)] if up else [(0, 1, 2), (0, 2, 3)]
        t.append(np.array([[base + a, base + b, base + c, mat] for a, b, c in tri], np.uint32))
        base += 4
    mats = np.array([[0.8, 0.3, 0.3, 0, 0, 0, 1.3, 0.1],
                     [0.3, 0.8, 0.3, 0, 0, 0, 1.5, 0.3],
                     [0.3, 0.3, 0.8, 0, 0, 0, 1.2, 0.05],
                     [0.7, 0.7, 0.7, 0, 0, 0, 1.8, 0.6],
                     [0.5, 0.5, 0.5, 0, 0, 0, 1.3, 0.9],
                     [0.0, 0.0, 0.0, 12, 11, 9, 1.3, 0.1]], np.float32)
    scene = Scene("lit_spheres", np.concatenate(v), np.concatenate(t))
    rays = camera_rays((0.0, 0.0, 35.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 65.0, res, res)
    return scene, mats, rays


def multi_scene_sizes(seed: int = 4, count: int = 64):
    """Triangle and ray counts of the uneven multi-scene batch (log-uniform)."""
    tris = [log_uniform(seed, 2 * i, 1024, 1 << 20) for i in range(count)]
    rays = [log_uniform(seed, 2 * i + 1, 4096, 1 << 20) for i in range(count)]
    return tris, rays


def icosphere_primary(res: int = 512):
    sc = icosphere()
    rays = camera_rays((0.0, 0.0, 3.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 65.0, res, res)
    return sc, rays

