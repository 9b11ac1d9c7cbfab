"""ctypes binding of the C-ABI (include/grt.h) and a Python mirror of the reference tracer.

``BatchRayTracer`` mirrors ``wf::cuda::batch_rt`` (rt/cuda/base.h:403-429) as the wavefront
steps use it: ``build`` a scene, ``use`` a ray-data object, ``compute_closest_hit`` /
``compute_any_hit`` over all of its rays, and ``interprete`` the reference's script commands
(``bvh type``, ``bvh max_tris`` from rt/cuda/base.cpp:134-153, ``raytracer`` from
rt/cuda/platform.cpp:102-131). Every call goes through libgrt.so; there is no Python or CPU
implementation of any traversal here. PyTorch is used only to hold device buffers.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import _libs

GRT_OK = 0
STATUS_NAMES = {0: "GRT_OK", 1: "GRT_ERR_INVALID_ARG", 2: "GRT_ERR_OOM", 3: "GRT_ERR_CUDA", 4: "GRT_ERR_TIMEOUT",
                5: "GRT_ERR_BVH_TOO_DEEP", 6: "GRT_ERR_NOT_BUILT", 7: "GRT_ERR_TRAVERSAL",
                8: "GRT_ERR_UNKNOWN_TRACER", 9: "GRT_ERR_NO_DEVICE", 10: "GRT_ERR_TOO_LARGE",
                11: "GRT_ERR_ABORTED"}
SPLIT = {"om": 0, "sm": 1, "sah": 2}
TRACERS = ("while-while", "persistent-while-while", "if-if", "persistent-if-if", "speculative-while-while",
           "persistent-speculative-while-while", "bvh4-speculative-while-while",
           "persistent-bvh4-speculative-while-while")
EXACT_TRACERS = TRACERS[:4]  # per-ray visit order of the reference: bit-identical results
ALPHA_TRACERS = tuple(t + "-alpha" for t in TRACERS)  # alpha-aware variants (set_alpha)


class GRTError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class BvhOpts(ctypes.Structure):
    _fields_ = [("split", ctypes.c_int), ("max_tris_per_node", ctypes.c_int), ("number_of_planes", ctypes.c_int),
                ("esc", ctypes.c_int)]


class BvhStats(ctypes.Structure):
    _fields_ = [("ref_nodes", ctypes.c_uint32), ("inner_nodes", ctypes.c_uint32), ("tri_records", ctypes.c_uint32),
                ("depth", ctypes.c_uint32), ("device_bytes", ctypes.c_uint64), ("build_ms", ctypes.c_double),
                ("flatten_ms", ctypes.c_double), ("upload_ms", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class LeafStats(ctypes.Structure):
    _fields_ = [("leaves", ctypes.c_uint32), ("min_tris", ctypes.c_int32), ("max_tris", ctypes.c_int32),
                ("avg_tris", ctypes.c_uint32), ("median_tris", ctypes.c_int32)]


class AlphaTexture(ctypes.Structure):
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("alpha", ctypes.c_void_p)]


class Tuning(ctypes.Structure):
    _fields_ = [("block_threads", ctypes.c_int), ("blocks_per_sm", ctypes.c_int), ("refill_threshold", ctypes.c_int),
                ("refill_period", ctypes.c_int), ("stack_entries", ctypes.c_int), ("spec_pend", ctypes.c_int),
                ("spec_exit", ctypes.c_int), ("spec_visits", ctypes.c_int)]


# grt_tuning fields a tuning-table entry may set (the rest of an entry names the tracer and tree)
TUNING_KEYS = tuple(k for k, _ in Tuning._fields_)


class PtParams(ctypes.Structure):
    _fields_ = [("max_bounces", ctypes.c_uint32), ("rr_start", ctypes.c_uint32), ("rr_continue", ctypes.c_float),
                ("eps", ctypes.c_float), ("seed", ctypes.c_uint64), ("mode", ctypes.c_int), ("use_graph", ctypes.c_int)]


PT_WAVEFRONT, PT_FUSED = 0, 1


class DirectParams(ctypes.Structure):
    _fields_ = [("samples", ctypes.c_uint32), ("mode", ctypes.c_uint32), ("seed", ctypes.c_uint64),
                ("sampling", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]


DL_WAVEFRONT, DL_FUSED = 0, 1
DL_SAMPLING = {"light": 0, "uniform": 1, "cosine": 2}  # GRT_DL_SAMPLE_*


TIMING_KINDS = ("trace", "trace_multi", "pathtrace", "direct", "adjoint", "tree", "rays")  # GRT_TIME_*


class Timing(ctypes.Structure):
    _fields_ = [("calls", ctypes.c_uint64 * len(TIMING_KINDS)), ("ms", ctypes.c_double * len(TIMING_KINDS))]


class Mesh(ctypes.Structure):
    _fields_ = [("vpos4", ctypes.c_void_p), ("nv", ctypes.c_uint32), ("tris4", ctypes.c_void_p), ("nt", ctypes.c_uint32)]


class RayBatch(ctypes.Structure):
    _fields_ = [("scene", ctypes.c_uint32), ("n", ctypes.c_uint32), ("rays_dev", ctypes.c_void_p),
                ("hits_dev", ctypes.c_void_p)]


class Camera(ctypes.Structure):
    """grt_camera: the fields of the reference's struct camera (libgi/camera.h:7-24)."""
    _fields_ = [("pos", ctypes.c_float * 3), ("dir", ctypes.c_float * 3), ("up", ctypes.c_float * 3),
                ("near_w", ctypes.c_float), ("near_h", ctypes.c_float)]


class Config(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("reserved", ctypes.c_uint32)]


_lib = None
P, U32, I, VP = ctypes.POINTER, ctypes.c_uint32, ctypes.c_int, ctypes.c_void_p

_PROTOS = {
    "grt_version": (I, []),
    "grt_create": (I, [P(Config), P(VP)]),
    "grt_destroy": (I, [VP]),
    "grt_last_error": (ctypes.c_char_p, [VP]),
    "grt_bvh_opts_default": (None, [P(BvhOpts)]),
    "grt_build": (I, [VP, VP, U32, VP, U32, P(BvhOpts)]),
    "grt_bvh_info": (I, [VP, P(BvhStats)]),
    "grt_export_bvh": (I, [VP, VP, VP, P(U32)]),
    "grt_host_bvh_build": (I, [VP, U32, VP, U32, P(BvhOpts), P(VP)]),
    "grt_host_bvh_info": (I, [VP, P(BvhStats)]),
    "grt_host_bvh_export": (I, [VP, VP, VP, P(U32)]),
    "grt_host_bvh_free": (None, [VP]),
    "grt_select_tracer": (I, [VP, ctypes.c_char_p]),
    "grt_set_tuning": (I, [VP, P(Tuning)]),
    "grt_get_tuning": (I, [VP, P(Tuning)]),
    "grt_trace": (I, [VP, VP, VP, U32, I, VP]),
    "grt_trace_host": (I, [VP, VP, VP, U32, I]),
    "grt_check": (I, [VP, VP, U32]),
    "grt_abort": (I, [VP]),
    "grt_set_traversal_counters": (I, [VP, VP]),
    "grt_compact_hits": (I, [VP, VP, U32, VP, VP, VP]),
    "grt_shadow_rays": (I, [VP, VP, VP, U32, P(ctypes.c_float), ctypes.c_float, VP, VP, VP]),
    "grt_set_materials": (I, [VP, VP, U32]),
    "grt_pt_params_default": (None, [P(PtParams)]),
    "grt_pathtrace": (I, [VP, P(PtParams), VP, VP, U32, U32, VP, VP, VP]),
    "grt_adjoint": (I, [VP, VP, VP, VP, U32, VP, U32, VP, VP, VP]),
    "grt_build_scenes": (I, [VP, VP, U32, P(BvhOpts)]),
    "grt_scene_info": (I, [VP, U32, P(BvhStats)]),
    "grt_export_scene_bvh": (I, [VP, U32, VP, VP, P(U32)]),
    "grt_trace_multi": (I, [VP, VP, U32, I, VP]),
    "grt_set_alpha": (I, [VP, VP, U32, VP, U32, VP, U32]),
    "grt_set_material_table": (I, [VP, VP, U32]),
    "grt_direct": (I, [VP, P(DirectParams), VP, U32, VP, VP]),
    "grt_hit_albedo": (I, [VP, U32, VP, U32, VP, VP]),
    "grt_set_bvh_cache": (I, [VP, ctypes.c_char_p]),
    "grt_bvh_cache_stats": (I, [VP, P(ctypes.c_uint64), P(ctypes.c_uint64)]),
    "grt_export_bvh_obj": (I, [VP, I, ctypes.c_char_p]),
    "grt_bvh_leaf_stats": (I, [VP, P(LeafStats)]),
    "grt_host_bvh_export_obj": (I, [VP, I, ctypes.c_char_p]),
    "grt_host_bvh_leaf_stats": (I, [VP, P(LeafStats)]),
    "grt_build_device": (I, [VP, VP, U32, VP, U32, U32, VP]),
    "grt_build_scenes_device": (I, [VP, VP, U32, U32, VP]),
    "grt_refit": (I, [VP, VP, U32, VP]),
    "grt_set_timing": (I, [VP, I]),
    "grt_timing_stats": (I, [VP, P(Timing), I]),
    "grt_incoherent_rays": (I, [VP, ctypes.c_float, ctypes.c_float, ctypes.c_uint64, VP, U32, VP]),
    "grt_camera_rays": (I, [VP, P(Camera), U32, U32, VP, I, ctypes.c_uint64, VP, VP]),
    "grt_set_device_builder": (I, [VP, I]),
    "grt_set_device_sah_planes": (I, [VP, U32]),
}


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        path = os.path.join(_libs.LIB_DIR, "libgrt.so")
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is missing: build it first (python -c 'import __graft_entry__ as g; g.build()')")
        L = ctypes.CDLL(path)
        for name, (res, args) in _PROTOS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _ptr(a) -> int:
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return a.data_ptr()  # torch tensor


def _check_cuda_tensor(t, name: str, cols: int):
    if not (hasattr(t, "is_cuda") and t.is_cuda and t.is_contiguous() and t.dim() == 2 and t.shape[1] == cols
            and t.element_size() == 4):
        raise ValueError(f"{name} must be a contiguous CUDA tensor of shape [n, {cols}] with 4-byte elements")


def make_opts(split="sah", max_tris=4, planes=16, esc=True) -> BvhOpts:
    return BvhOpts(SPLIT[split] if isinstance(split, str) else int(split), int(max_tris), int(planes), int(bool(esc)))


class HostBVH:
    """The product builder run on the host only (grt_host_bvh_*): reference-layout nodes."""

    def __init__(self, vpos, tris, **opts):
        v = np.ascontiguousarray(vpos, np.float32)
        t = np.ascontiguousarray(tris, np.uint32)
        h = VP()
        o = make_opts(**opts)
        st = lib().grt_host_bvh_build(_ptr(v), v.shape[0], _ptr(t), t.shape[0], ctypes.byref(o), ctypes.byref(h))
        if st != GRT_OK:
            raise GRTError(st, "host BVH build failed")
        self.h = h
        s = BvhStats()
        lib().grt_host_bvh_info(self.h, ctypes.byref(s))
        self.stats = s.as_dict()

    def export(self):
        nodes = np.zeros((self.stats["ref_nodes"], 14), np.uint32)
        index = np.zeros(self.stats["tri_records"], np.uint32)
        root = U32()
        lib().grt_host_bvh_export(self.h, _ptr(nodes), _ptr(index), ctypes.byref(root))
        return nodes, index, int(root.value)

    def export_obj(self, max_depth: int, path: str):
        st = lib().grt_host_bvh_export_obj(self.h, int(max_depth), str(path).encode())
        if st != GRT_OK:
            raise GRTError(st, f"cannot write {path}")

    def leaf_stats(self) -> dict:
        s = LeafStats()
        st = lib().grt_host_bvh_leaf_stats(self.h, ctypes.byref(s))
        if st != GRT_OK:
            raise GRTError(st, "no leaf statistics for this tree")
        return {k: getattr(s, k) for k, _ in s._fields_}

    def __del__(self):
        try:
            lib().grt_host_bvh_free(self.h)
        except Exception:
            pass


class RayData:
    """Device ray and hit buffers in the reference's CUDA layout (wf::cuda::raydata,
    rt/cuda/base.h:328-351): rays float32 [n, 8], hits float32 [n, 4] (ref as uint32 bits)."""

    def __init__(self, rays, hits=None):
        import torch
        self.rays = rays
        self.hits = hits if hits is not None else torch.empty((rays.shape[0], 4), dtype=torch.float32,
                                                              device=rays.device)

    @property
    def n(self) -> int:
        return int(self.rays.shape[0])


class BatchRayTracer:
    """One traversal context on one GPU (a grt_ctx)."""

    def __init__(self, device: int = 0):
        cfg = Config(device, 0)
        h = VP()
        st = lib().grt_create(ctypes.byref(cfg), ctypes.byref(h))
        if st != GRT_OK:
            raise GRTError(st, "grt_create failed")
        self.ctx = h
        self.device = device
        self.bvh_type = "sah"         # `bvh type`
        self.bvh_max_tris_per_node = 4  # `bvh max_tris`
        self.bvh_planes = 16            # `bvh sah <planes>` of the CPU tracer
        self.use_incoherence = False    # `incoherence r1 r2`
        self.incoherence_r1 = self.incoherence_r2 = 0.0
        self.rd: RayData | None = None
        self.tracer = TRACERS[0]

    # -- helpers ------------------------------------------------------------------------
    def _check(self, st: int):
        if st != GRT_OK:
            msg = lib().grt_last_error(self.ctx)
            raise GRTError(st, msg.decode() if msg else "")

    def close(self):
        if getattr(self, "ctx", None):
            lib().grt_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- wf::batch_ray_tracer surface -----------------------------------------------------
    def interprete(self, command: str) -> bool:
        """Script commands of the CUDA tracer and platform (`incoherence r1 r2`, `bvh type`,
        `bvh max_tris`, rt/cuda/base.cpp:119-153; `raytracer`, rt/cuda/platform.cpp:102-131)
        and of the CPU tracer (`bvh om|sm|sah <planes>|triangles single|multiple <n>|statistics|
        export <depth> <file>`, rt/cpu/bvh2.cpp:192-241); returns False for unknown ones."""
        words = command.split()
        if words and words[0] == "incoherence":
            if len(words) != 3:
                raise ValueError('"incoherence" requires exactly two positive float values')
            r1, r2 = float(words[1]), float(words[2])
            if r1 < 0 or r2 < 0:
                raise ValueError('"incoherence" requires exactly two positive float values')
            if r1 != 0 or r2 != 0:  # as the reference: 0 0 leaves the setting unchanged
                self.use_incoherence, self.incoherence_r1, self.incoherence_r2 = True, r1, r2
            return True
        if len(words) == 3 and words[:2] == ["bvh", "type"]:
            if words[2] not in SPLIT:
                raise ValueError('"bvh type" must be one of "sm", "om", "sah"')
            self.bvh_type = words[2]
            return True
        if len(words) == 3 and words[:2] == ["bvh", "max_tris"]:
            self.bvh_max_tris_per_node = int(words[2])
            return True
        if len(words) == 2 and words[0] == "raytracer":
            self.select(words[1])
            return True
        if len(words) >= 2 and words[0] == "bvh":
            sub = words[1:]
            if sub in (["om"], ["sm"]):
                self.bvh_type = sub[0]
                return True
            if len(sub) == 2 and sub[0] == "sah":
                self.bvh_type, self.bvh_planes = "sah", int(sub[1])
                return True
            if sub == ["triangles", "single"]:
                self.bvh_max_tris_per_node = 1
                return True
            if len(sub) == 3 and sub[:2] == ["triangles", "multiple"]:
                self.bvh_max_tris_per_node = int(sub[2])
                return True
            if sub == ["statistics"]:
                st = self.leaf_stats()
                print(f"number of leaf nodes: {st['leaves']}")
                print(f"minimum triangles per node: {st['min_tris']}")
                print(f"maximum triangles per node: {st['max_tris']}")
                print(f"average triangles per node: {st['avg_tris']}")
                print(f"median of triangles per node: {st['median_tris']}")
                return True
            if len(sub) == 3 and sub[0] == "export":
                self.export_obj(int(sub[1]), sub[2])
                print(f"bvh exported to {sub[2]}")
                return True
        return False

    def set_bvh_cache(self, directory):
        """On-disk cache of built trees (grt_set_bvh_cache); None switches it off."""
        self._check(lib().grt_set_bvh_cache(self.ctx, directory.encode() if directory else None))

    def cache_stats(self):
        hits, misses = ctypes.c_uint64(), ctypes.c_uint64()
        self._check(lib().grt_bvh_cache_stats(self.ctx, ctypes.byref(hits), ctypes.byref(misses)))
        return int(hits.value), int(misses.value)

    def export_obj(self, max_depth: int, path: str):
        """The tree's boxes above max_depth as OBJ (the reference's `bvh export`)."""
        self._check(lib().grt_export_bvh_obj(self.ctx, int(max_depth), str(path).encode()))

    def leaf_stats(self) -> dict:
        """The reference's `bvh statistics` figures of the current tree."""
        st = LeafStats()
        self._check(lib().grt_bvh_leaf_stats(self.ctx, ctypes.byref(st)))
        return {k: getattr(st, k) for k, _ in st._fields_}

    def select(self, name: str):
        self._check(lib().grt_select_tracer(self.ctx, name.encode()))
        self.tracer = name

    def build(self, vpos, tris, split=None, max_tris=None, planes=None, esc=True) -> dict:
        self._refit_key = None  # autograd.closest_hits(builder="refit") builds anew
        v = np.ascontiguousarray(vpos, np.float32)
        t = np.ascontiguousarray(tris, np.uint32)
        o = make_opts(split or self.bvh_type, max_tris or self.bvh_max_tris_per_node, planes or self.bvh_planes, esc)
        self._check(lib().grt_build(self.ctx, _ptr(v), v.shape[0], _ptr(t), t.shape[0], ctypes.byref(o)))
        return self.info()

    DEVICE_BUILDERS = {"default": 0, "lbvh": 1, "ploc": 2, "sah": 3}

    def set_device_builder(self, method: str, planes: int | None = None):
        """grt_set_device_builder: "sah", "ploc", "lbvh" or "default" (SAH); `planes`:
        grt_set_device_sah_planes (candidate planes of the SAH builder, 1..256)."""
        self._check(lib().grt_set_device_builder(self.ctx, self.DEVICE_BUILDERS[method]))
        if planes is not None:
            self._check(lib().grt_set_device_sah_planes(self.ctx, int(planes)))

    def build_device(self, vpos, tris, max_tris=None, stream=None) -> dict:
        """The GPU builder (grt_build_device) on CUDA tensors: vpos float32 [nv, 4], tris
        int32/uint32 [nt, 4]. Returns the build statistics."""
        self._refit_key = None  # autograd.closest_hits(builder="refit") builds anew
        _check_cuda_tensor(vpos, "vpos", 4)
        _check_cuda_tensor(tris, "tris", 4)
        self._check(lib().grt_build_device(self.ctx, _ptr(vpos), int(vpos.shape[0]), _ptr(tris), int(tris.shape[0]),
                                           int(max_tris or self.bvh_max_tris_per_node), VP(stream or 0)))
        return self.info()

    def set_timing(self, enabled: bool = True):
        """grt_set_timing: per-call device timers (the reference's wavefront step timers)."""
        self._check(lib().grt_set_timing(self.ctx, int(bool(enabled))))

    def timing_stats(self, reset: bool = False) -> dict:
        """grt_timing_stats: {kind: (calls, device ms)} since the last reset."""
        t = Timing()
        self._check(lib().grt_timing_stats(self.ctx, ctypes.byref(t), int(bool(reset))))
        return {k: (int(t.calls[i]), float(t.ms[i])) for i, k in enumerate(TIMING_KINDS)}

    def incoherent_rays(self, n: int, seed: int = 1234, stream=None, r1=None, r2=None):
        """grt_incoherent_rays: a CUDA tensor [n, 8] of the `incoherence r1 r2` test rays of the
        built scene (the radii of the last `incoherence` command unless given)."""
        import torch
        rays = torch.empty((int(n), 8), dtype=torch.float32, device=f"cuda:{self.device}")
        a = self.incoherence_r1 if r1 is None else r1
        b = self.incoherence_r2 if r2 is None else r2
        self._check(lib().grt_incoherent_rays(self.ctx, float(a), float(b), int(seed), _ptr(rays), int(n),
                                              VP(stream or 0)))
        return rays

    def camera_rays(self, pos, dir, up, near_w, near_h, w: int, h: int, rays=None, offsets=None, jitter=False,
                    seed: int = 0, stream=None):
        """grt_camera_rays: the w x h camera rays of the primary-ray step as cam_ray computes them
        (libgi/camera.cpp:11-28), into `rays` (a CUDA tensor [w h, 8], allocated if None).
        offsets: a CUDA tensor [w h, 2] of sub-pixel offsets in [-0.5, 0.5), or None (then PCG
        jitter from `seed` when `jitter`, else pixel centres)."""
        import torch
        n = int(w) * int(h)
        if rays is None:
            rays = torch.empty((n, 8), dtype=torch.float32, device=f"cuda:{self.device}")
        _check_cuda_tensor(rays, "rays", 8)
        if rays.shape[0] < n:
            raise ValueError("rays holds fewer than w * h rays")
        if offsets is not None:
            _check_cuda_tensor(offsets, "offsets", 2)
            if offsets.shape[0] < n:
                raise ValueError("offsets holds fewer than w * h pairs")
        cam = Camera((ctypes.c_float * 3)(*pos), (ctypes.c_float * 3)(*dir), (ctypes.c_float * 3)(*up),
                     float(near_w), float(near_h))
        self._check(lib().grt_camera_rays(self.ctx, ctypes.byref(cam), int(w), int(h),
                                          _ptr(offsets) if offsets is not None else None, int(bool(jitter)),
                                          int(seed), _ptr(rays), VP(stream or 0)))
        return rays

    def refit(self, vpos, stream=None):
        """grt_refit: the built tree refitted to new vertex positions, a CUDA tensor float32
        [nv, 4] of the built scene's vertex count."""
        _check_cuda_tensor(vpos, "vpos", 4)
        self._check(lib().grt_refit(self.ctx, _ptr(vpos), int(vpos.shape[0]), VP(stream or 0)))

    def set_material_table(self, mats):
        """Materials for direct lighting (grt_set_material_table): float32 [m, 8] = albedo rgb,
        emission rgb, ior, roughness. Triangles with an emitting material are the lights."""
        m = np.ascontiguousarray(mats, np.float32).reshape(-1, 8)
        self._check(lib().grt_set_material_table(self.ctx, _ptr(m), m.shape[0]))

    def direct(self, rays, framebuffer, samples, mode=DL_FUSED, seed=0, stream=None, sampling="light"):
        """Direct lighting (grt_direct) of CUDA rays [n, 8], accumulated into the CUDA frame
        buffer [n, 4] (radiance sum, sample count); sampling "light", "uniform" or "cosine"
        (the reference direct-wf's `sampling` setting)."""
        p = DirectParams(int(samples), int(mode), int(seed), DL_SAMPLING[sampling], 0)
        self._check(lib().grt_direct(self.ctx, ctypes.byref(p), _ptr(rays), int(rays.shape[0]), _ptr(framebuffer),
                                     VP(stream or 0)))

    def hit_albedo(self, rays, framebuffer, mode=DL_FUSED, stream=None):
        """primary-wf's shading (grt_hit_albedo): framebuffer [n, 4] += (albedo of the closest
        hit's material, 1) for CUDA rays [n, 8]."""
        self._check(lib().grt_hit_albedo(self.ctx, int(mode), _ptr(rays), int(rays.shape[0]), _ptr(framebuffer),
                                         VP(stream or 0)))

    def set_alpha(self, tc, mat_tex, textures):
        """Texture data of the alpha-aware tracers (grt_set_alpha): tc float32 [nv, 2] per vertex
        of the built scene, mat_tex int32 [n_materials] (texture index or -1), textures: list of
        float32 [height, width] alpha arrays. set_alpha(None, None, None) clears it."""
        if mat_tex is None:
            self._check(lib().grt_set_alpha(self.ctx, None, 0, None, 0, None, 0))
            return
        tc = np.ascontiguousarray(tc, np.float32)
        mt = np.ascontiguousarray(mat_tex, np.int32)
        tex = [np.ascontiguousarray(t, np.float32) for t in textures]
        arr = (AlphaTexture * max(1, len(tex)))(*[AlphaTexture(t.shape[1], t.shape[0], t.ctypes.data) for t in tex])
        self._check(lib().grt_set_alpha(self.ctx, _ptr(tc), tc.shape[0], _ptr(mt), mt.shape[0], arr, len(tex)))

    def use(self, rd: RayData):
        self.rd = rd

    def compute_closest_hit(self):
        self._run(False)

    def compute_any_hit(self):
        self._run(True)

    def _run(self, any_hit: bool):
        import torch
        if self.rd is None:
            raise RuntimeError("use() a RayData first")
        stream = torch.cuda.current_stream(self.rd.rays.device).cuda_stream
        self.trace(self.rd.rays, self.rd.hits, any_hit, stream)
        self.check(stream)  # the reference synchronises after every launch (rt/cuda/tracers.cu:67-68)

    # -- direct access ------------------------------------------------------------------
    def trace(self, rays, hits, any_hit=False, stream=None, n=None):
        n = int(rays.shape[0]) if n is None else int(n)
        self._check(lib().grt_trace(self.ctx, _ptr(rays), _ptr(hits), n, int(any_hit), VP(stream or 0)))

    def set_traversal_counters(self, counters=None):
        """counters: a CUDA int64 tensor of 3 (rays, inner nodes, triangle tests) or None."""
        self._check(lib().grt_set_traversal_counters(self.ctx, _ptr(counters) if counters is not None else None))

    def check(self, stream=None, timeout_ms: int = 0):
        self._check(lib().grt_check(self.ctx, VP(stream or 0), timeout_ms))

    def abort(self):
        """grt_abort: the context's persistent kernels stop taking work until the next check();
        callable from another thread while this one waits in check()."""
        self._check(lib().grt_abort(self.ctx))

    def trace_host(self, rays: np.ndarray, any_hit=False, hits: np.ndarray | None = None) -> np.ndarray:
        r = np.ascontiguousarray(rays, np.float32)
        out = hits if hits is not None else np.zeros((r.shape[0], 4), np.float32)
        self._check(lib().grt_trace_host(self.ctx, _ptr(r), _ptr(out), r.shape[0], int(any_hit)))
        return out

    def info(self) -> dict:
        s = BvhStats()
        self._check(lib().grt_bvh_info(self.ctx, ctypes.byref(s)))
        return s.as_dict()

    def export_bvh(self):
        info = self.info()
        nodes = np.zeros((info["ref_nodes"], 14), np.uint32)
        index = np.zeros(info["tri_records"], np.uint32)
        root = U32()
        self._check(lib().grt_export_bvh(self.ctx, _ptr(nodes), _ptr(index), ctypes.byref(root)))
        return nodes, index, int(root.value)

    def set_tuning(self, **kw):
        t = Tuning()
        self._check(lib().grt_get_tuning(self.ctx, ctypes.byref(t)))
        for k, v in kw.items():
            setattr(t, k, int(v))
        self._check(lib().grt_set_tuning(self.ctx, ctypes.byref(t)))

    def get_tuning(self) -> dict:
        t = Tuning()
        self._check(lib().grt_get_tuning(self.ctx, ctypes.byref(t)))
        return {k: getattr(t, k) for k, _ in t._fields_}

    # -- ray generation and path tracing -------------------------------------------------
    def compact_hits(self, hits, indices, count, stream=None):
        self._check(lib().grt_compact_hits(self.ctx, _ptr(hits), int(hits.shape[0]), _ptr(indices), _ptr(count),
                                           VP(stream or 0)))

    def shadow_rays(self, rays, hits, light, eps, out_rays, count, stream=None):
        lt = (ctypes.c_float * 3)(*[float(x) for x in light])
        self._check(lib().grt_shadow_rays(self.ctx, _ptr(rays), _ptr(hits), int(rays.shape[0]), lt,
                                          ctypes.c_float(eps), _ptr(out_rays), _ptr(count), VP(stream or 0)))

    def set_materials(self, albedo):
        a = np.ascontiguousarray(albedo, np.float32)
        self._check(lib().grt_set_materials(self.ctx, _ptr(a) if a.size else None, int(a.size)))

    @staticmethod
    def pt_params(**kw) -> PtParams:
        p = PtParams()
        lib().grt_pt_params_default(ctypes.byref(p))
        for k, v in kw.items():
            setattr(p, k, v)
        return p

    def pathtrace(self, params: PtParams, prim_rays, prim_hits, n_paths, results, bounce_hits=None, stream=None):
        self._check(lib().grt_pathtrace(self.ctx, ctypes.byref(params), _ptr(prim_rays), _ptr(prim_hits),
                                        int(prim_rays.shape[0]), int(n_paths), _ptr(results),
                                        _ptr(bounce_hits) if bounce_hits is not None else None, VP(stream or 0)))

    def adjoint(self, rays, hits, grad_hits, grad_vpos=None, grad_rays=None, vpos=None, stream=None):
        """grt_adjoint: grad_hits [n, 3] = (dL/dt, dL/dbeta, dL/dgamma); grad_vpos [nv, 3] is added to,
        grad_rays [n, 8] written. vpos: [nv, 3] or [nv, 4] float32 device tensor, or None for the
        built scene's vertices."""
        vstride = 0 if vpos is None else int(vpos.shape[1])
        self._check(lib().grt_adjoint(self.ctx, _ptr(rays), _ptr(hits), _ptr(grad_hits), int(rays.shape[0]),
                                      _ptr(vpos) if vpos is not None else None, vstride,
                                      _ptr(grad_vpos) if grad_vpos is not None else None,
                                      _ptr(grad_rays) if grad_rays is not None else None, VP(stream or 0)))

    # -- many scenes in one launch ----------------------------------------------------------
    def build_scenes(self, scenes, **opts) -> list:
        """scenes: list of (vpos float32 [nv, 4], tris uint32 [nt, 4]). Returns per-scene stats."""
        self._refit_key = None  # autograd.closest_hits(builder="refit") builds anew
        keep = [(np.ascontiguousarray(v, np.float32), np.ascontiguousarray(t, np.uint32)) for v, t in scenes]
        arr = (Mesh * len(keep))(*[Mesh(_ptr(v), v.shape[0], _ptr(t), t.shape[0]) for v, t in keep])
        o = make_opts(**{"split": self.bvh_type, "max_tris": self.bvh_max_tris_per_node, **opts})
        self._check(lib().grt_build_scenes(self.ctx, arr, len(keep), ctypes.byref(o)))
        out = []
        for i in range(len(keep)):
            st = BvhStats()
            self._check(lib().grt_scene_info(self.ctx, i, ctypes.byref(st)))
            out.append(st.as_dict())
        return out

    def build_scenes_device(self, scenes, max_tris=None, stream=None) -> list:
        """The GPU builder over a scene set (grt_build_scenes_device): scenes is a list of
        (vpos CUDA float32 [nv, 4], tris CUDA int32/uint32 [nt, 4]). Returns per-scene stats."""
        self._refit_key = None  # autograd.closest_hits(builder="refit") builds anew
        for v, t in scenes:
            _check_cuda_tensor(v, "vpos", 4)
            _check_cuda_tensor(t, "tris", 4)
        arr = (Mesh * len(scenes))(*[Mesh(_ptr(v), int(v.shape[0]), _ptr(t), int(t.shape[0])) for v, t in scenes])
        self._check(lib().grt_build_scenes_device(self.ctx, arr, len(scenes), int(max_tris or self.bvh_max_tris_per_node),
                                                  VP(stream or 0)))
        out = []
        for i in range(len(scenes)):
            st = BvhStats()
            self._check(lib().grt_scene_info(self.ctx, i, ctypes.byref(st)))
            out.append(st.as_dict())
        return out

    def export_scene_bvh(self, scene: int, ref_nodes: int, tri_records: int):
        nodes = np.zeros((ref_nodes, 14), np.uint32)
        index = np.zeros(tri_records, np.uint32)
        root = U32()
        self._check(lib().grt_export_scene_bvh(self.ctx, scene, _ptr(nodes), _ptr(index), ctypes.byref(root)))
        return nodes, index, int(root.value)

    def trace_multi(self, batches, any_hit=False, stream=None):
        """batches: list of (scene, rays tensor [n, 8], hits tensor [n, 4])."""
        arr = (RayBatch * len(batches))(*[RayBatch(s, int(r.shape[0]), _ptr(r), _ptr(h)) for s, r, h in batches])
        self._check(lib().grt_trace_multi(self.ctx, arr, len(batches), int(any_hit), VP(stream or 0)))
