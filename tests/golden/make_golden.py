"""Generates the golden fixtures in this directory from the REFERENCE's own CPU tracer.

Needs oracle/_ref/libref_bbvh.so, which oracle/build_ref.sh compiles from the unmodified
reference sources (rt/cpu/bvh2.cpp and its headers). For every scene in the list below it
stores, per builder configuration of cases.BUILDERS, the SHA-256 of the reference's BVH
(bbvh_node array, index array, root) and, for the default CUDA configuration (SAH, 16 planes,
4 triangles per leaf, early split clipping), the reference's closest hits of the scene's rays
and its any-hit answers for a set of rays with finite t_max.

The alpha-aware case (cases.alpha_scene) is stored the same way from the reference's
alpha-aware tracer (binary_bvh_tracer<indexed, esc on, true>).

Run from the repository root:  python tests/golden/make_golden.py  (or ... make_golden.py alpha)
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

import __graft_entry__ as ge  # noqa: E402
import cases  # noqa: E402


def bvh_digest(nodes: np.ndarray, index: np.ndarray, root: int) -> np.ndarray:
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(nodes, np.uint32).tobytes())
    h.update(np.ascontiguousarray(index, np.uint32).tobytes())
    h.update(np.uint32(root).tobytes())
    return np.frombuffer(h.digest(), np.uint8).copy()


def array_digest(a: np.ndarray) -> np.ndarray:
    return np.frombuffer(hashlib.sha256(np.ascontiguousarray(a).tobytes()).digest(), np.uint8).copy()


def scenes():
    """name -> (vpos, tris, closest rays, rays stored in the fixture?, any-hit rays)."""
    ge.load_package()
    from illum_rt_gb300 import workloads as wl
    out = {}
    sc, rays = wl.heightfield_primary()
    out["heightfield"] = (sc.vpos, sc.tris, rays, False,
                          cases.random_rays(101, 4096, (0, 0, 0.0), (1, 1, 0.3), tmax_scale=0.5))
    sc = wl.spheres()
    rays = wl.camera_rays((0.0, 0.0, 35.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 65.0, 256, 256)
    out["spheres"] = (sc.vpos, sc.tris, rays, False,
                      cases.random_rays(102, 8192, (-10, -10, -10), (10, 10, 10), tmax_scale=4.0))
    v, t = cases.kat_scene()
    kr = cases.kat_rays()
    out["kat"] = (v, t, kr, True, kr)
    sc = wl.soup(11, 3000)
    lo, hi = sc.bounds()
    out["soup3000"] = (sc.vpos, sc.tris, cases.random_rays(103, 8192, lo, hi), True,
                       cases.random_rays(104, 8192, lo, hi, tmax_scale=2.0))
    sc = wl.icosphere(levels=3)
    rays = wl.camera_rays((0.0, 0.0, 3.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 65.0, 128, 128)
    out["icosphere3"] = (sc.vpos, sc.tris, rays, False,
                         cases.random_rays(105, 4096, (-1, -1, -1), (1, 1, 1), tmax_scale=1.0))
    return out


def main():
    orc = ge.load_oracle()
    if not orc.ref_available():
        sys.exit("oracle/_ref/libref_bbvh.so missing: run oracle/build_ref.sh (needs the reference sources)")
    for name, (v, t, rays, store_rays, any_rays) in scenes().items():
        data = {"vpos_digest": array_digest(v), "tris_digest": array_digest(t), "rays_digest": array_digest(rays)}
        for bname, opts in cases.BUILDERS:
            ref = orc.ReferenceBVH(v, t, **opts)
            data["bvh_" + bname] = bvh_digest(ref.nodes(), ref.index(), ref.root)
            data["nodes_" + bname] = np.int64(ref.nodes().shape[0])
        ref = orc.ReferenceBVH(v, t, **dict(cases.BUILDERS[0][1]))
        depth = orc.OracleBVH(v, t, **dict(cases.BUILDERS[0][1])).depth()
        assert depth <= 23, f"{name}: depth {depth} would overflow the reference's 25-entry stack"
        data["closest"] = ref.closest(rays)
        data["any_rays"] = any_rays
        data["any_occluded"] = ref.any(any_rays)
        if store_rays:
            data["rays"] = rays
        if name == "kat":
            data["vpos"] = v
            data["tris"] = t
        path = os.path.join(HERE, f"golden_{name}.npz")
        np.savez_compressed(path, **data)
        hits = int((data["closest"][:, 0] < cases.FLT_MAX).sum())
        print(f"{name}: {rays.shape[0]} rays, {hits} hits, {int(data['any_occluded'].sum())} occluded "
              f"of {any_rays.shape[0]}, {os.path.getsize(path)} bytes")


def main_alpha():
    """The alpha-aware case: the reference's binary_bvh_tracer<indexed, esc on, true>."""
    orc = ge.load_oracle()
    v, t, tc, mat_tex, textures = cases.alpha_scene()
    rays, any_rays = cases.alpha_rays()
    alpha = orc.AlphaSet(tc, mat_tex, textures)
    ref = orc.ReferenceAlphaBVH(v, t, alpha)
    data = {"vpos_digest": array_digest(v), "tris_digest": array_digest(t), "tc_digest": array_digest(tc),
            "texels_digest": array_digest(alpha.texels), "rays_digest": array_digest(rays),
            "any_rays_digest": array_digest(any_rays),
            "closest": ref.closest(rays), "any_occluded": ref.any(any_rays)}
    path = os.path.join(HERE, "golden_alpha.npz")
    np.savez_compressed(path, **data)
    hits = int((data["closest"][:, 0] < cases.FLT_MAX).sum())
    print(f"alpha: {rays.shape[0]} rays, {hits} hits, {int(data['any_occluded'].sum())} occluded "
          f"of {any_rays.shape[0]}, {os.path.getsize(path)} bytes")


TOOL_DEPTHS = (1, 4, 9)


def main_tools():
    """The reference tracer's `bvh export <depth> <file>` and `bvh statistics` outputs for every
    golden scene (default CUDA build): SHA-256 of each exported OBJ text and the printed lines."""
    import tempfile
    orc = ge.load_oracle()
    data = {}
    for name, (v, t, _, _, _) in scenes().items():
        ref = orc.ReferenceBVH(v, t, **dict(cases.BUILDERS[0][1]))
        for d in TOOL_DEPTHS:
            with tempfile.TemporaryDirectory() as tmp:
                path = os.path.join(tmp, "bvh.obj")
                orc.ref_bvh_command(ref, f"export {d} {path}")
                with open(path, "rb") as f:
                    data[f"obj_{name}_{d}"] = array_digest(np.frombuffer(f.read(), np.uint8))
        try:
            text = orc.ref_bvh_command(ref, "statistics")
        except Exception:  # the reference's median reads past the end for two leaves
            text = ""
        data[f"stats_{name}"] = np.frombuffer(text.encode(), np.uint8).copy()
    path = os.path.join(HERE, "golden_bvh_tools.npz")
    np.savez_compressed(path, **data)
    print(f"bvh tools: {len(data)} entries, {os.path.getsize(path)} bytes")


if __name__ == "__main__":
    if sys.argv[1:] == ["alpha"]:
        main_alpha()
    elif sys.argv[1:] == ["tools"]:
        main_tools()
    else:
        main()
        main_alpha()
        main_tools()
