"""ctypes access to the oracle (oracle.cpp) and to the reference build (oracle/_ref).

Test infrastructure only: the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module, as the checker. The product never does.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libref_bbvh.so")

SPLIT = {"om": 0, "sm": 1, "sah": 2}
_libs: dict[str, ctypes.CDLL] = {}


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _load(path: str, prefix: str) -> ctypes.CDLL:
    if path in _libs:
        return _libs[path]
    if not os.path.exists(path):
        raise RuntimeError(f"{path} missing: run oracle/build.py")
    lib = ctypes.CDLL(path)
    getattr(lib, prefix + "build").restype = ctypes.c_void_p
    getattr(lib, prefix + "build").argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_uint32,
                                               ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    for fn in ("root", "num_nodes", "num_index"):
        getattr(lib, prefix + fn).restype = ctypes.c_uint32
        getattr(lib, prefix + fn).argtypes = [ctypes.c_void_p]
    for fn in ("get_nodes", "get_index", "free"):
        getattr(lib, prefix + fn).argtypes = [ctypes.c_void_p] + ([ctypes.c_void_p] if fn != "free" else [])
    _libs[path] = lib
    return lib


def ref_available() -> bool:
    return os.path.exists(REF_SO)


SAMPLING = {"light": 0, "uniform": 1, "cosine": 2}  # grt_direct_params::sampling


class _BVHBase:
    prefix = ""

    def __init__(self, lib, vpos, tris, esc=True, split="sah", max_tris=4, planes=16):
        self.lib = lib
        self._v = np.ascontiguousarray(vpos, np.float32)
        self._t = np.ascontiguousarray(tris, np.uint32)
        self.h = getattr(lib, self.prefix + "build")(_p(self._v), self._v.shape[0], _p(self._t), self._t.shape[0],
                                                     int(esc), SPLIT[split], max_tris, planes)

    def _fn(self, name):
        return getattr(self.lib, self.prefix + name)

    @property
    def root(self) -> int:
        return int(self._fn("root")(self.h))

    def nodes(self) -> np.ndarray:
        """uint32 [n, 14]: box_l.lo, box_l.hi, box_r.lo, box_r.hi (float bits), link_l, link_r."""
        n = self._fn("num_nodes")(self.h)
        out = np.zeros((n, 14), np.uint32)
        self._fn("get_nodes")(self.h, _p(out))
        return out

    def index(self) -> np.ndarray:
        n = self._fn("num_index")(self.h)
        out = np.zeros(n, np.uint32)
        self._fn("get_index")(self.h, _p(out))
        return out

    def __del__(self):
        try:
            self._fn("free")(ctypes.c_void_p(self.h))
        except Exception:
            pass


class OracleBVH(_BVHBase):
    """The oracle restatement: reference builder + bbvh traversal."""
    prefix = "orc_"

    def __init__(self, vpos, tris, **kw):
        lib = _load(ORACLE_SO, "orc_")
        lib.orc_depth.restype = ctypes.c_uint32
        lib.orc_depth.argtypes = [ctypes.c_void_p]
        lib.orc_closest.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p,
                                    ctypes.c_void_p, ctypes.c_int]
        lib.orc_any.argtypes = lib.orc_closest.argtypes
        lib.orc_failed.argtypes = [ctypes.c_void_p]
        super().__init__(lib, vpos, tris, **kw)
        if lib.orc_failed(self.h):
            raise RuntimeError("oracle BVH build found no split (non-finite input?)")

    def depth(self) -> int:
        return int(self.lib.orc_depth(self.h))

    def closest(self, rays, threads=0, counts=False):
        """Returns (hits float32[n,4] with ref in the last column as uint32 bits, counts|None)."""
        rays = np.ascontiguousarray(rays, np.float32)
        n = rays.shape[0]
        out = np.zeros((n, 4), np.float32)
        cnt = np.zeros((n, 3), np.uint32) if counts else None
        self.lib.orc_closest(self.h, _p(rays), n, _p(out), _p(cnt) if counts else None, threads)
        return out, cnt

    def shadow_rays(self, rays, hits, light, eps=1e-4):
        """Shadow rays of the valid hits, in ray order (float32 [count, 8])."""
        rays = np.ascontiguousarray(rays, np.float32)
        hits = np.ascontiguousarray(hits, np.float32)
        out = np.zeros((rays.shape[0], 8), np.float32)
        lt = np.asarray(light, np.float32)
        f = self.lib.orc_shadow_rays
        f.restype = ctypes.c_uint32
        f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p,
                      ctypes.c_float, ctypes.c_void_p]
        cnt = f(self.h, _p(rays), _p(hits), rays.shape[0], _p(lt), eps, _p(out))
        return out[:cnt]

    def pathtrace(self, prim_rays, prim_hits, n_paths, max_bounces=5, rr_start=3, rr_continue=0.8, eps=1e-4, seed=0,
                  albedo=None, bounce_hits=False, threads=0, totals=None):
        """Diffuse paths as grt_pathtrace defines them: (results uint32 [n, 4] with the radiance as
        float bits in column 0, bounce hit records float32 [n, max_bounces, 4] or None). `totals`,
        a uint64 array of 3, receives (bounce rays, inner-node visits, triangle tests)."""
        prim_rays = np.ascontiguousarray(prim_rays, np.float32)
        prim_hits = np.ascontiguousarray(prim_hits, np.float32)
        alb = np.ascontiguousarray(albedo if albedo is not None else np.zeros(0), np.float32)
        res = np.zeros((n_paths, 4), np.uint32)
        bh = np.zeros((n_paths, max_bounces, 4), np.float32) if bounce_hits else None
        f = self.lib.orc_pathtrace
        f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint64,
                      ctypes.c_uint32, ctypes.c_uint32, ctypes.c_float, ctypes.c_float, ctypes.c_uint64,
                      ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        f(self.h, _p(prim_rays), _p(prim_hits), prim_rays.shape[0], n_paths, max_bounces, rr_start, rr_continue, eps,
          seed, _p(alb) if alb.size else None, alb.size, _p(res), _p(bh) if bh is not None else None,
          _p(totals) if totals is not None else None, threads)
        return res, bh

    def any(self, rays, threads=0, counts=False):
        rays = np.ascontiguousarray(rays, np.float32)
        n = rays.shape[0]
        occ = np.zeros(n, np.uint8)
        cnt = np.zeros((n, 3), np.uint32) if counts else None
        self.lib.orc_any(self.h, _p(rays), n, _p(occ), _p(cnt) if counts else None, threads)
        return occ, cnt

    def direct(self, rays, mats, samples, seed=0, threads=0, sampling="light"):
        """Direct lighting as grt_direct defines it: float32 [n, 4] frame buffer (radiance sum,
        sample count) for camera rays [n, 8] and materials [m, 8] (albedo rgb, emission rgb,
        ior, roughness); sampling "light", "uniform" or "cosine"."""
        rays = np.ascontiguousarray(rays, np.float32)
        mats = np.ascontiguousarray(mats, np.float32)
        fb = np.zeros((rays.shape[0], 4), np.float32)
        f = self.lib.orc_direct
        f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_uint32,
                      ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_int]
        f(self.h, _p(rays), rays.shape[0], _p(mats), mats.shape[0], samples, seed, SAMPLING[sampling], _p(fb),
          threads)
        return fb

    def hit_albedo(self, rays, mats, fb=None):
        """add_hitpoint_albedo (rt/cuda/kernels.cu:170-197), untextured: fb + (albedo of the
        closest hit's material, 1), (0, 0, 0, 1) for a miss; materials beyond the table have the
        reference's default material (albedo 0)."""
        mats = np.ascontiguousarray(mats, np.float32).reshape(-1, 8)
        h, _ = self.closest(rays)
        add = np.zeros((h.shape[0], 4), np.float32)
        add[:, 3] = 1.0
        hit = h[:, 0] != np.float32(3.4028234663852886e38)
        mat = self._t[h[hit, 3].view(np.uint32), 3]
        known = mat < mats.shape[0]
        alb = np.zeros((mat.shape[0], 3), np.float32)
        alb[known] = mats[mat[known], 0:3]
        add[hit, 0:3] = alb
        base = np.zeros_like(add) if fb is None else np.asarray(fb, np.float32)
        return (base + add).astype(np.float32)

    def set_alpha(self, alpha):
        """Alpha-aware tracing from now on (alpha: an AlphaSet), or off with None."""
        f = self.lib.orc_set_alpha
        f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_uint32,
                      ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32]
        if alpha is None:
            f(self.h, None, 0, None, 0, None, None, 0)
            return
        self._alpha = alpha  # keeps the arrays alive for the call
        f(self.h, _p(alpha.tc), alpha.tc.shape[0], _p(alpha.mat_tex), alpha.mat_tex.shape[0], _p(alpha.tex_wh),
          _p(alpha.texels), alpha.tex_wh.shape[0])


class AlphaSet:
    """Texture data of the alpha-aware tracers: tc float32 [nv, 2], mat_tex int32 [n_materials]
    (texture index or -1), textures: list of float32 [h, w] alpha arrays."""

    def __init__(self, tc, mat_tex, textures):
        self.tc = np.ascontiguousarray(tc, np.float32)
        self.mat_tex = np.ascontiguousarray(mat_tex, np.int32)
        self.textures = [np.ascontiguousarray(t, np.float32) for t in textures]
        self.tex_wh = np.ascontiguousarray([[t.shape[1], t.shape[0]] for t in self.textures] or np.zeros((0, 2)),
                                           np.uint32).reshape(-1, 2)
        self.texels = np.ascontiguousarray(np.concatenate([t.ravel() for t in self.textures])
                                           if self.textures else np.zeros(1), np.float32)


class ReferenceBVH(_BVHBase):
    """The reference's own binary_bvh_tracer, compiled from its sources into oracle/_ref."""
    prefix = "ref_"

    def __init__(self, vpos, tris, **kw):
        lib = _load(REF_SO, "ref_")
        lib.ref_closest.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_int]
        lib.ref_any.argtypes = lib.ref_closest.argtypes
        super().__init__(lib, vpos, tris, **kw)

    def closest(self, rays, threads=0):
        rays = np.ascontiguousarray(rays, np.float32)
        out = np.zeros((rays.shape[0], 4), np.float32)
        self.lib.ref_closest(self.h, _p(rays), rays.shape[0], _p(out), threads)
        return out

    def any(self, rays, threads=0):
        rays = np.ascontiguousarray(rays, np.float32)
        occ = np.zeros(rays.shape[0], np.uint8)
        self.lib.ref_any(self.h, _p(rays), rays.shape[0], _p(occ), threads)
        return occ


def ref_bvh_command(ref: "ReferenceBVH", args: str) -> str:
    """Runs the reference tracer's `bvh <args>` command on `ref` and returns its stdout."""
    f = ref.lib.ref_bvh_command
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int]
    buf = ctypes.create_string_buffer(1 << 16)
    if not f(ref.h, args.encode(), buf, len(buf)):
        raise RuntimeError(f"the reference did not take 'bvh {args}'")
    return buf.value.decode()


class ReferenceAlphaBVH(ReferenceBVH):
    """The reference's alpha-aware tracer (binary_bvh_tracer<indexed, esc on, true>, SAH)."""

    def __init__(self, vpos, tris, alpha: AlphaSet, max_tris=4, planes=16):
        lib = _load(REF_SO, "ref_")
        lib.ref_closest.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_int]
        lib.ref_any.argtypes = lib.ref_closest.argtypes
        f = lib.ref_build_alpha
        f.restype = ctypes.c_void_p
        f.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p,
                      ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32,
                      ctypes.c_int, ctypes.c_int]
        self.lib = lib
        self._v = np.ascontiguousarray(vpos, np.float32)
        self._t = np.ascontiguousarray(tris, np.uint32)
        self._alpha = alpha
        self.h = f(_p(self._v), self._v.shape[0], _p(self._t), self._t.shape[0], _p(alpha.tc), _p(alpha.mat_tex),
                   alpha.mat_tex.shape[0], _p(alpha.tex_wh), _p(alpha.texels), alpha.tex_wh.shape[0], max_tris, planes)


def max_threads() -> int:
    lib = _load(ORACLE_SO, "orc_")
    return int(lib.orc_max_threads())


def _orc():
    return _load(ORACLE_SO, "orc_")


def fixed_hits64(vpos3, tris4, rays6, refs):
    """(t, beta, gamma) in double for each ray against its given triangle."""
    vpos3 = np.ascontiguousarray(vpos3, np.float64)
    rays6 = np.ascontiguousarray(rays6, np.float64)
    tris4 = np.ascontiguousarray(tris4, np.uint32)
    refs = np.ascontiguousarray(refs, np.uint32)
    out = np.zeros((refs.shape[0], 3), np.float64)
    f = _orc().orc_fixed_hits64
    f.argtypes = [ctypes.c_void_p] * 4 + [ctypes.c_uint64, ctypes.c_void_p]
    f(_p(vpos3), _p(tris4), _p(rays6), _p(refs), refs.shape[0], _p(out))
    return out


def adjoint64(vpos3, tris4, rays6, refs, grad3):
    """FP64 analytic gradients: (dL/dvpos [nv, 3], dL/d(o, d) [n, 6]) for grad3 = (dt, dbeta, dgamma)."""
    vpos3 = np.ascontiguousarray(vpos3, np.float64)
    rays6 = np.ascontiguousarray(rays6, np.float64)
    tris4 = np.ascontiguousarray(tris4, np.uint32)
    refs = np.ascontiguousarray(refs, np.uint32)
    grad3 = np.ascontiguousarray(grad3, np.float64)
    gv = np.zeros_like(vpos3)
    gr = np.zeros((refs.shape[0], 6), np.float64)
    f = _orc().orc_adjoint64
    f.argtypes = [ctypes.c_void_p] * 5 + [ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p]
    f(_p(vpos3), _p(tris4), _p(rays6), _p(refs), _p(grad3), refs.shape[0], _p(gv), _p(gr))
    return gv, gr


# ---- the oracle's own copy of the benchmark workload (scenes.cpp) --------------------------

def spheres_scene(seed=2, count=256, slices=32, stacks=16, cext=10.0, rmin=0.2, rmax=1.5):
    """(vpos float32 [nv, 4], tris uint32 [nt, 4]) of the UV-sphere scene."""
    v = np.zeros((count * (stacks + 1) * slices, 4), np.float32)
    t = np.zeros((count * 2 * slices * stacks, 4), np.uint32)
    f = _orc().orc_scene_spheres
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_float, ctypes.c_float,
                  ctypes.c_float, ctypes.c_void_p, ctypes.c_void_p]
    if f(seed, count, slices, stacks, cext, rmin, rmax, _p(v), _p(t)) != 0:
        raise ValueError("slices and stacks must divide 32 and 16")
    return v, t


def camera_rays(pos, look, up, fovy_deg, w, h, tmin=1e-4):
    """float32 [w h, 8] pixel-centre pinhole rays, (o, t_min, d, t_max)."""
    r = np.zeros((w * h, 8), np.float32)
    p, lk, u = (np.asarray(x, np.float32) for x in (pos, look, up))
    f = _orc().orc_camera_rays
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_float, ctypes.c_uint32,
                  ctypes.c_uint32, ctypes.c_float, ctypes.c_void_p]
    if f(_p(p), _p(lk), _p(u), fovy_deg, w, h, tmin, _p(r)) != 0:
        raise ValueError("field of view outside (0, 180) degrees")
    return r


def spheres_primary(res=1024):
    """The benchmark workload: the 262,144-triangle sphere scene and its res x res primary rays
    from (0, 0, 35) towards the origin, 65 degrees vertical field of view."""
    v, t = spheres_scene()
    return v, t, camera_rays((0.0, 0.0, 35.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 65.0, res, res)


def cam_rays(pos, dir, up, near_w, near_h, w, h, offsets=None, jitter=False, seed=0):
    """float32 [w h, 8] camera rays in cam_ray's float arithmetic (scenes.cpp orc_cam_rays)."""
    r = np.zeros((w * h, 8), np.float32)
    p, d, u = (np.asarray(x, np.float32) for x in (pos, dir, up))
    off = np.ascontiguousarray(offsets, np.float32) if offsets is not None else None
    f = _orc().orc_cam_rays
    f.restype = None
    f.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_float, ctypes.c_float, ctypes.c_uint32, ctypes.c_uint32,
                                          ctypes.c_void_p, ctypes.c_int, ctypes.c_uint64, ctypes.c_void_p]
    f(_p(p), _p(d), _p(u), near_w, near_h, w, h, _p(off) if off is not None else None, int(bool(jitter)), seed, _p(r))
    return r


def ref_cam_rays(pos, dir, up, near_w, near_h, w, h, offsets=None, jitter=False, seed=0):
    """The same rays from the reference's own cam_ray (oracle/_ref/libref_sampling.so), or None
    where the reference build is absent."""
    path = os.path.join(HERE, "_ref", "libref_sampling.so")
    if not os.path.exists(path):
        return None
    lib = ctypes.CDLL(path)
    r = np.zeros((w * h, 8), np.float32)
    p, d, u = (np.asarray(x, np.float32) for x in (pos, dir, up))
    off = np.ascontiguousarray(offsets, np.float32) if offsets is not None else None
    f = lib.refs_cam_rays_offsets
    f.restype = None
    f.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_float, ctypes.c_float, ctypes.c_int, ctypes.c_int,
                                          ctypes.c_void_p, ctypes.c_int, ctypes.c_uint64, ctypes.c_void_p]
    f(_p(p), _p(d), _p(u), near_w, near_h, w, h, _p(off) if off is not None else None, int(bool(jitter)), seed, _p(r))
    return r
