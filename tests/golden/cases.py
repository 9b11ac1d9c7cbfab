"""Definitions of the golden cases: scenes, rays and builder options.

``make_golden.py`` runs the reference's own CPU tracer (oracle/_ref, built from the reference
sources) on these cases and stores its outputs next to this file; the tests check the oracle,
the product builder and the GPU kernels against them.
"""
from __future__ import annotations

import numpy as np

FLT_MAX = np.float32(3.4028234663852886e38)
INF = np.float32(np.inf)
NAN = np.float32(np.nan)


def kat_scene():
    """Known-answer scene (15 triangles): a flat 3x3-vertex grid at z = 0 (8 triangles), two
    exact duplicates of grid triangle 0 (equal-t ties), two zero-area triangles, a small
    triangle hovering at z = 0.5, a steep triangle and a far-away one."""
    v = []
    for j in range(3):
        for i in range(3):
            v.append((0.5 * i, 0.5 * j, 0.0))
    t = []
    for j in range(2):
        for i in range(2):
            a = 3 * j + i
            t.append((a, a + 1, a + 4))
            t.append((a, a + 4, a + 3))
    t.append(t[0])                       # duplicate of triangle 0
    t.append((t[0][1], t[0][2], t[0][0]))  # duplicate with rotated vertex order
    nv = len(v)
    v += [(0.2, 0.2, 0.25), (0.4, 0.4, 0.25), (0.6, 0.6, 0.25)]  # collinear: zero area
    t.append((nv, nv + 1, nv + 2))
    t.append((nv, nv, nv + 1))  # repeated vertex: zero area
    nv = len(v)
    v += [(0.1, 0.1, 0.5), (0.3, 0.1, 0.5), (0.1, 0.3, 0.5)]
    t.append((nv, nv + 1, nv + 2))
    nv = len(v)
    v += [(0.9, 0.0, 0.0), (0.9, 1.0, 0.0), (0.9, 0.5, 0.8)]
    t.append((nv, nv + 1, nv + 2))
    nv = len(v)
    v += [(10.0, 10.0, 10.0), (11.0, 10.0, 10.0), (10.0, 11.0, 10.0)]
    t.append((nv, nv + 1, nv + 2))
    vpos = np.zeros((len(v), 4), np.float32)
    vpos[:, :3] = np.asarray(v, np.float32)
    vpos[:, 3] = 1
    tris = np.zeros((len(t), 4), np.uint32)
    tris[:, :3] = np.asarray(t, np.uint32)
    return vpos, tris


def _ray(o, d, tmin=np.float32(1e-4), tmax=FLT_MAX):
    return [o[0], o[1], o[2], tmin, d[0], d[1], d[2], tmax]


def kat_rays():
    """Hand-built rays: centre, back-face, edges, vertices, exact t_min / t_max boundaries,
    rays parallel to the plane, axis-aligned rays whose origin lies on a box face (0 * inf
    slab products), zero / NaN / subnormal / negative-zero directions, huge origins, and a
    grid of axis-aligned rays through every vertex and edge of the flat grid."""
    r = []
    down, up = (0.0, 0.0, -1.0), (0.0, 0.0, 1.0)
    r.append(_ray((0.35, 0.15, 1.0), down))             # plain hit
    r.append(_ray((0.35, 0.15, -1.0), up))              # back face
    r.append(_ray((2.0, 2.0, 1.0), down))               # miss
    r.append(_ray((0.25, 0.25, 1.0), down))             # shared diagonal edge
    r.append(_ray((0.0, 0.0, 1.0), down))               # grid vertex
    r.append(_ray((0.0, 0.25, 1.0), down))              # on the x = 0 face of the root box
    r.append(_ray((-1.0, 0.25, 0.0), (1.0, 0.0, 0.0)))  # in the plane of the grid
    r.append(_ray((0.35, 0.15, 1.0), down, np.float32(1.0)))                 # t == t_min
    r.append(_ray((0.35, 0.15, 1.0), down, np.float32(0.0), np.float32(1.0)))  # t == t_max
    r.append(_ray((0.35, 0.15, 1.0), down, np.float32(0.0), np.float32(np.nextafter(np.float32(1), np.float32(2)))))
    r.append(_ray((0.35, 0.15, 1.0), down, -INF, INF))
    r.append(_ray((0.35, 0.15, 1.0), (0.0, 0.0, 0.0)))  # zero direction
    r.append(_ray((0.35, 0.15, 1.0), (NAN, 0.0, -1.0)))  # NaN direction
    r.append(_ray((0.35, 0.15, 1.0), (1e-40, 0.0, -1.0)))  # subnormal component
    r.append(_ray((0.35, 0.15, 1.0), (-0.0, -0.0, -1.0)))  # negative zeros
    r.append(_ray((1e30, 0.15, 1.0), (-1.0, 0.0, -1e-30)))  # huge origin
    r.append(_ray((0.15, 0.15, 2.0), down))             # hovering triangle in front of the grid
    r.append(_ray((0.15, 0.15, 0.4), down))             # origin between hovering triangle and grid
    r.append(_ray((0.15, 0.15, 0.4), up))               # hovering triangle from below
    r.append(_ray((0.4, 0.1, 1.0), (0.0, 0.0, -1.0), np.float32(0.0), NAN))   # NaN t_max
    r.append(_ray((0.4, 0.1, 1.0), (0.0, 0.0, -1.0), NAN, FLT_MAX))           # NaN t_min
    r.append(_ray((0.5, 0.5, 0.3), (1.0, 0.0, -0.1)))   # towards the steep triangle
    r.append(_ray((10.2, 10.2, 20.0), down))            # far triangle
    r.append(_ray((0.3, 0.3, 0.0), (0.0, 0.0, -1.0)))   # origin on the surface
    # the same boundaries for a direction with no zero component (the packed slab test's rays)
    tilt = (0.01, 0.02, -1.0)
    r.append(_ray((0.4, 0.1, 1.0), tilt, np.float32(0.0), NAN))                # NaN t_max
    r.append(_ray((0.4, 0.1, 1.0), tilt, NAN, FLT_MAX))                        # NaN t_min
    r.append(_ray((0.4, 0.1, 1.0), tilt, np.float32(2.0), np.float32(1.0)))   # t_min > t_max
    r.append(_ray((0.4, 0.1, 1.0), tilt, np.float32(0.0), np.float32(0.0)))   # t_max = 0
    r.append(_ray((0.4, 0.1, 1.0), tilt, -INF, INF))                           # unbounded both ways
    r.append(_ray((0.35, 0.15, -1.0), tilt, np.float32(-10.0), FLT_MAX))       # hits behind the origin
    r.append(_ray((0.3, 0.3, 0.0), tilt, np.float32(-1.0), FLT_MAX))           # hit at t = 0
    r.append(_ray((0.3, 0.3, 1e-7), tilt, np.float32(-1.0), FLT_MAX))          # hit just below t = 0
    r.append(_ray((0.35, 0.15, 1.0), tilt, np.float32(1.0), FLT_MAX))          # t near t_min
    for y in np.arange(-0.25, 1.3, 0.125):
        for x in np.arange(-0.25, 1.3, 0.125):
            r.append(_ray((x, y, 1.0), down))
    return np.asarray(r, np.float32)


def random_rays(seed: int, n: int, lo, hi, tmax_scale=None):
    """Rays from points in the box [lo, hi] towards random directions (any-hit cases when
    tmax_scale is given: t_max is uniform in [0, tmax_scale])."""
    g = np.random.default_rng(seed)
    lo, hi = np.asarray(lo, np.float64), np.asarray(hi, np.float64)
    o = lo + (hi - lo) * g.random((n, 3))
    d = g.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = np.zeros((n, 8), np.float32)
    r[:, 0:3] = o
    r[:, 3] = 1e-4
    r[:, 4:7] = d
    r[:, 7] = FLT_MAX if tmax_scale is None else tmax_scale * g.random(n)
    return r


# (name, builder options) pairs whose BVHs are pinned by hash for every scene.
BUILDERS = [
    ("sah16_4_esc", dict(split="sah", max_tris=4, planes=16, esc=True)),
    ("sah16_4", dict(split="sah", max_tris=4, planes=16, esc=False)),
    ("sah8_1_esc", dict(split="sah", max_tris=1, planes=8, esc=True)),
    ("sm_4_esc", dict(split="sm", max_tris=4, planes=1, esc=True)),
    ("om_2", dict(split="om", max_tris=2, planes=1, esc=False)),
    ("sah64_2", dict(split="sah", max_tris=2, planes=64, esc=False)),  # the benchmark's tuned tree
]


def alpha_scene():
    """Alpha-aware case: two stacked 33x33-vertex grids over [0,1]^2 (z = 0 and z = 0.1, the upper
    one with a height ripple), 4,096 triangles, texture coordinates spanning [-1.5, 2.5] (several
    wraps, negative values), and four materials by triangle index mod 4: no texture (opaque), an
    8x8 checker of alpha 0 / 1, a 16x4 ramp whose texels include exactly 0.5 (the threshold is
    strict), and a fully transparent 3x5 texture.
    Returns (vpos, tris, tc [nv, 2], mat_tex [4], textures)."""
    n = 33
    xs = np.linspace(0.0, 1.0, n, dtype=np.float32)
    X, Y = np.meshgrid(xs, xs)
    layers = []
    for z0, amp in ((0.0, 0.0), (0.1, 0.03)):
        Z = z0 + amp * np.sin(9.0 * X) * np.cos(7.0 * Y)
        layers.append(np.stack([X, Y, Z.astype(np.float32)], -1).reshape(-1, 3))
    v3 = np.concatenate(layers)
    vpos = np.ones((v3.shape[0], 4), np.float32)
    vpos[:, :3] = v3
    t = []
    for layer in range(2):
        base = layer * n * n
        for j in range(n - 1):
            for i in range(n - 1):
                a = base + j * n + i
                t.append((a, a + 1, a + n + 1))
                t.append((a, a + n + 1, a + n))
    tris = np.zeros((len(t), 4), np.uint32)
    tris[:, :3] = np.asarray(t, np.uint32)
    tris[:, 3] = np.arange(len(t)) % 4
    tc = (v3[:, :2] * 4.0 - 1.5).astype(np.float32)
    tc[n * n:] = (tc[n * n:] * 0.75 + 0.3).astype(np.float32)
    checker = ((np.arange(8)[:, None] + np.arange(8)[None, :]) % 2).astype(np.float32)
    ramp = np.tile(np.linspace(0.2, 0.8, 16, dtype=np.float32), (4, 1))
    ramp[:, 5] = 0.5
    ramp[1, :] = 0.5
    clear = np.zeros((5, 3), np.float32)
    return vpos, tris, tc, np.array([-1, 0, 1, 2], np.int32), [checker, ramp, clear]


def alpha_rays():
    """Closest-hit rays: a 96x96 pinhole frame looking down at the grids plus 4,096 random rays;
    any-hit rays: 4,096 random rays with finite t_max."""
    o = np.array([0.5, -0.4, 1.2], np.float32)
    u, w = np.meshgrid(np.linspace(0.05, 0.95, 96), np.linspace(0.05, 0.95, 96))
    target = np.stack([u, w, np.zeros_like(u)], -1).reshape(-1, 3)
    d = target - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    cam = np.zeros((d.shape[0], 8), np.float32)
    cam[:, 0:3] = o
    cam[:, 3] = 1e-4
    cam[:, 4:7] = d
    cam[:, 7] = FLT_MAX
    rnd = random_rays(106, 4096, (0.0, 0.0, -0.2), (1.0, 1.0, 0.3))
    return np.concatenate([cam, rnd]), random_rays(107, 4096, (0.0, 0.0, -0.2), (1.0, 1.0, 0.3), tmax_scale=0.6)
