"""Wavefront OBJ (+ MTL) scenes in the library's layouts.

The reference loads scenes through assimp (libgi/scene.cpp), which this image does not have; a
scene reaches the tracer as float4 vertex positions (x, y, z, 1) and uint4 triangles (a, b, c,
material id), rt/cuda/base.cpp:48-68, and direct lighting reads per material the albedo,
emission, index of refraction and roughness (libgi/material.h:144-151). ``load_obj`` reads the
geometry and materials of an OBJ file into exactly those arrays:

* ``v x y z [w]`` vertices; ``f`` faces with 1-based or negative (relative) indices in any of the
  forms ``i``, ``i/t``, ``i//n``, ``i/t/n``; polygons are split into a fan around their first
  vertex, as assimp's triangulation does for convex faces;
* ``usemtl name`` selects the material of the following faces; names are numbered in order of
  first use, faces before any ``usemtl`` get material 0 named ``""``;
* ``mtllib file`` loads each material as the reference's importer converts assimp's
  (libgi/scene.cpp:323-334): albedo = ``Kd`` if its luma exceeds 1e-4, else ``Ks``, raised to
  the power 2.2; emission = ``Ke``; roughness = sqrt(2 / (``Ns`` + 2))
  (roughness_from_exponent, libgi/material.h:12-14); ior = ``Ni``, with 1.0 read as 1.3; missing
  values take the reference's defaults (albedo 0, emission 0, ior 1.3, roughness 0.1).

Texture coordinates, normals, groups and other statements are skipped.
"""
from __future__ import annotations

import os

import numpy as np

DEFAULT_MATERIAL = (0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 1.3, 0.1)  # libgi/material.h:144-151


def _luma(c) -> float:  # libgi/color.h:4-6
    return 0.212671 * c[0] + 0.715160 * c[1] + 0.072169 * c[2]


def _mtl(path: str) -> dict:
    raw, cur = {}, None
    with open(path) as f:
        for line in f:
            w = line.split()
            if not w or w[0].startswith("#"):
                continue
            if w[0] == "newmtl":
                cur = " ".join(w[1:])
                raw[cur] = {}
            elif cur is not None and w[0] in ("Kd", "Ks", "Ke") and len(w) >= 4:
                raw[cur][w[0]] = [float(x) for x in w[1:4]]
            elif cur is not None and w[0] in ("Ns", "Ni") and len(w) >= 2:
                raw[cur][w[0]] = float(w[1])
    out = {}
    for name, r in raw.items():
        m = list(DEFAULT_MATERIAL)
        kd, ks = r.get("Kd", [0.0] * 3), r.get("Ks", [0.0] * 3)
        alb = np.asarray(kd if _luma(kd) > 1e-4 else ks, np.float32)
        m[0:3] = np.power(alb, np.float32(2.2)).tolist()
        m[3:6] = r.get("Ke", [0.0] * 3)
        if "Ns" in r:
            m[7] = float(np.sqrt(np.float32(2.0) / (np.float32(r["Ns"]) + np.float32(2.0))))
        if "Ni" in r:
            m[6] = 1.3 if r["Ni"] == 1.0 else r["Ni"]
        out[name] = m
    return out


def load_obj(path: str):
    """(vpos float32 [nv, 4], tris uint32 [nt, 4], material names, materials float32 [m, 8])."""
    verts: list[tuple[float, float, float]] = []
    tris: list[tuple[int, int, int, int]] = []
    names: list[str] = []
    ids: dict[str, int] = {}
    library: dict[str, list] = {}
    current = None
    base = os.path.dirname(os.path.abspath(path))

    def material_id() -> int:
        name = "" if current is None else current
        if name not in ids:
            ids[name] = len(names)
            names.append(name)
        return ids[name]

    def index(tok: str, line_no: int) -> int:
        k = int(tok.split("/")[0])
        k = k - 1 if k > 0 else len(verts) + k
        if not 0 <= k < len(verts):
            raise ValueError(f"{path}:{line_no}: vertex index {tok} out of range")
        return k

    with open(path) as f:
        for line_no, line in enumerate(f, 1):
            w = line.split()
            if not w or w[0].startswith("#"):
                continue
            if w[0] == "v":
                verts.append((float(w[1]), float(w[2]), float(w[3])))
            elif w[0] == "f":
                if len(w) < 4:
                    raise ValueError(f"{path}:{line_no}: a face needs three vertices")
                idx = [index(t, line_no) for t in w[1:]]
                m = material_id()
                for k in range(1, len(idx) - 1):
                    tris.append((idx[0], idx[k], idx[k + 1], m))
            elif w[0] == "usemtl":
                current = " ".join(w[1:])
            elif w[0] == "mtllib":
                for lib_name in w[1:]:
                    p = os.path.join(base, lib_name)
                    if os.path.exists(p):
                        library.update(_mtl(p))
    vpos = np.ones((len(verts), 4), np.float32)
    if verts:
        vpos[:, :3] = np.asarray(verts, np.float32)
    t = np.asarray(tris, np.uint32).reshape(-1, 4)
    mats = np.asarray([library.get(n, DEFAULT_MATERIAL) for n in names], np.float32).reshape(-1, 8)
    return vpos, t, names, mats
