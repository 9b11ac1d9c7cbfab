"""The sampling, ray-setup and shading helpers of the path tracer and of direct lighting, pinned to
the reference's own code (CPU).

The library's helpers (csrc/pt_math.cuh, csrc/dl_math.cuh) are compiled here for the host
(tests/ptmath_probe.cpp; on the device they are the same explicitly rounded operations, which
the GPU path-tracing tests check bit for bit through whole paths) and compared with the
reference's functions compiled from its sources (oracle/_ref/libref_sampling.so):

* bit for bit: the PCG32 stream (rng_pcg, libgi/random.h:59-96), align and
  flip_normals_to_ray (libgi/util.h:212-225), fresnel_dielectric and tan2_theta
  (libgi/util.h:91-106, 141-160), luma (libgi/color.h:4-6), the GGX terms ggx_d and ggx_g1
  (libgi/material.cpp:237-260, the same code as rt/cuda/bounce.cu:298-313);
* within a stated bound: sin and cos of 2 pi u, which the library evaluates with its own
  polynomial (sincos_turns) where the reference calls sinf / cosf of a float angle, and through it
  the cosine- and uniform-hemisphere samples (libgi/sampling.h:13-36); the pinhole camera rays,
  which the library's workload generator computes in double and rounds once where cam_ray
  (libgi/camera.cpp:11-28) computes in float.
"""
import ctypes
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_SO = os.path.join(ROOT, "oracle", "_ref", "libref_sampling.so")
U32 = ctypes.c_uint32


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


@pytest.fixture(scope="module")
def ptm(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("ptm") / "libptm.so")
    subprocess.run(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off",
                    "-I" + os.path.join(ROOT, "illum-rt_gb300", "csrc"), "-x", "c++",
                    os.path.join(ROOT, "tests", "ptmath_probe.cpp"), "-o", out], check=True)
    return ctypes.CDLL(out)


@pytest.fixture(scope="module")
def ref(pkg):
    if not os.path.exists(REF_SO):
        pytest.skip("reference sampling harness not built (reference sources absent)")
    return ctypes.CDLL(REF_SO)


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def test_sincos_turns_error_bound(ptm):
    """sin and cos of 2 pi u for every u = k 2^-24 in [0, 1) within 2.5e-7 of the double values
    (measured maximum 1.99e-7 = 2^-22.26, about 1.7 ulp at 1). The error is absolute: near the
    zeros of sin and cos the polynomial of the remaining angle (up to pi/2) cancels, so no
    relative bound holds there."""
    u = (np.arange(1 << 24, dtype=np.float64) / (1 << 24)).astype(np.float32)
    s, c = np.zeros_like(u), np.zeros_like(u)
    ptm.ptm_sincos_turns(_p(u), U32(u.size), _p(s), _p(c))
    a = 2 * np.pi * u.astype(np.float64)
    assert np.abs(s - np.sin(a)).max() <= 2.5e-7
    assert np.abs(c - np.cos(a)).max() <= 2.5e-7
    # exact at the quadrant starts
    q = np.array([0.0, 0.25, 0.5, 0.75], np.float32)
    qs, qc = np.zeros_like(q), np.zeros_like(q)
    ptm.ptm_sincos_turns(_p(q), U32(4), _p(qs), _p(qc))
    assert qs.tolist() == [0.0, 1.0, -0.0, -1.0] and qc.tolist() == [1.0, -0.0, -1.0, 0.0]


@pytest.mark.parametrize("seq", [0, 1, 7, 12345, (1 << 32) + 5, (1 << 63) - 1, 0xDEADBEEFCAFEF00D])
def test_pcg_stream_bit_exact(ptm, ref, seq):
    n = 4096
    w1, w2 = np.zeros(n, np.uint32), np.zeros(n, np.uint32)
    f1, f2 = np.zeros(n, np.float32), np.zeros(n, np.float32)
    ptm.ptm_pcg(ctypes.c_uint64(seq), U32(n), _p(w1), _p(f1))
    ref.refs_pcg(ctypes.c_uint64(seq), U32(n), _p(w2), _p(f2))
    assert (w1 == w2).all()
    assert (_bits(f1) == _bits(f2)).all() and f1.max() < 1.0


def _unit(g, n):
    v = g.normal(size=(n, 3))
    return (v / np.linalg.norm(v, axis=1, keepdims=True)).astype(np.float32)


def test_align_and_facing_normal_bit_exact(ptm, ref):
    g = np.random.default_rng(5)
    n = 200_000
    axis = _unit(g, n)
    axis[:6] = [[0, 0, 1], [0, 0, -1], [0, 0, 0.0], [0, 0, -0.0], [1, 0, 0], [0, -1, 0]]
    axis[6:12, 2] = -0.0
    v = _unit(g, n)
    v[:, 2] = np.abs(v[:, 2])
    a, b = np.zeros((n, 3), np.float32), np.zeros((n, 3), np.float32)
    ptm.ptm_align(_p(v), _p(axis), U32(n), _p(a))
    ref.refs_align(_p(v), _p(axis), U32(n), _p(b))
    assert (_bits(a) == _bits(b)).all()
    # facing normal: normalise(cross(b - a, c - a)), flipped when it faces along the ray
    p0, p1, p2 = (g.normal(size=(n, 3)).astype(np.float32) * 5 for _ in range(3))
    d = _unit(g, n)
    ptm.ptm_facing_normal(_p(p0), _p(p1), _p(p2), _p(d), U32(n), _p(a))
    ref.refs_facing_normal(_p(p0), _p(p1), _p(p2), _p(d), U32(n), _p(b))
    assert (_bits(a) == _bits(b)).all()


def test_fresnel_tan2_luma_bit_exact(ptm, ref):
    cos = np.concatenate([np.linspace(-1.2, 1.2, 4801), [0.0, -0.0, 1.0, -1.0, 1e-30, -1e-30]]).astype(np.float32)
    iors = [1.0, 1.3, 1.5, 2.4, 0.7]
    for m in iors:
        for t in iors:
            im, it = np.full_like(cos, m), np.full_like(cos, t)
            a, b = np.zeros_like(cos), np.zeros_like(cos)
            ptm.ptm_fresnel(_p(cos), _p(im), _p(it), U32(cos.size), _p(a))
            ref.refs_fresnel(_p(cos), _p(im), _p(it), U32(cos.size), _p(b))
            assert (_bits(a) == _bits(b)).all(), (m, t)
    a, b = np.zeros_like(cos), np.zeros_like(cos)
    ptm.ptm_tan2_theta(_p(cos), U32(cos.size), _p(a))
    ref.refs_tan2_theta(_p(cos), U32(cos.size), _p(b))
    assert (_bits(a) == _bits(b)).all()
    rgb = np.random.default_rng(2).random((10000, 3)).astype(np.float32) * 20
    a, b = np.zeros(10000, np.float32), np.zeros(10000, np.float32)
    ptm.ptm_luma(_p(rgb), U32(10000), _p(a))
    ref.refs_luma(_p(rgb), U32(10000), _p(b))
    assert (_bits(a) == _bits(b)).all()


def test_ggx_terms_bit_exact(ptm, ref):
    g = np.random.default_rng(4)
    cos = np.concatenate([g.uniform(-0.2, 1.0, 200_000), [0.0, -0.0, 1.0, 1e-30, 1e-20, 0.5]]).astype(np.float32)
    rough = np.concatenate([g.uniform(0.0, 1.0, 200_000), [0.1, 0.0, 1.0, 0.5, 0.05, 0.0]]).astype(np.float32)
    for name in ("ggx_d", "ggx_g1"):
        a, b = np.zeros_like(cos), np.zeros_like(cos)
        getattr(ptm, "ptm_" + name)(_p(cos), _p(rough), U32(cos.size), _p(a))
        getattr(ref, "refs_" + name)(_p(cos), _p(rough), U32(cos.size), _p(b))
        assert (_bits(a) == _bits(b)).all(), name


def test_hemisphere_samples_within_bound_of_reference(ptm, ref):
    """Cosine-weighted samples: x and y within 2.5e-7 of the exact values (the reference's own
    sinf / cosf of a rounded float angle: up to 4.2e-7 measured), so within 7e-7 of the
    reference's; z = sqrt(1 - x^2 - y^2) carries the same cancellation near the horizon in both
    (maximum error 7.8e-5 for each, measured), and the library's z error never exceeds the
    reference's maximum. Uniform-hemisphere samples within 1e-6 of the reference's."""
    g = np.random.default_rng(1)
    n = 2_000_000
    u0, u1 = g.random(n).astype(np.float32), g.random(n).astype(np.float32)
    u0[:4], u1[:4] = [0.0, 0.999999940, 0.5, 0.25], [0.0, 0.999999940, 0.25, 0.75]
    a, b = np.zeros((n, 3), np.float32), np.zeros((n, 3), np.float32)
    ptm.ptm_cosine_sample(_p(u0), _p(u1), U32(n), _p(a))
    ref.refs_cosine_sample(_p(u0), _p(u1), U32(n), _p(b))
    x0, x1 = u0.astype(np.float64), u1.astype(np.float64)
    exact = np.stack([np.sqrt(x0) * np.cos(2 * np.pi * x1), np.sqrt(x0) * np.sin(2 * np.pi * x1),
                      np.sqrt(np.maximum(0.0, 1.0 - x0))], 1)
    err_a, err_b = np.abs(a - exact), np.abs(b - exact)
    assert err_a[:, :2].max() <= 2.5e-7
    assert err_b[:, :2].max() <= 5e-7
    assert np.abs(a[:, :2].astype(np.float64) - b[:, :2]).max() <= 7e-7
    assert err_a[:, 2].max() <= err_b[:, 2].max() * 1.01 + 1e-9
    assert np.abs(a[:, 2].astype(np.float64) - b[:, 2]).max() <= 1e-4
    ptm.ptm_uniform_hemisphere(_p(u0), _p(u1), U32(n), _p(a))
    ref.refs_uniform_hemisphere(_p(u0), _p(u1), U32(n), _p(b))
    assert np.abs(a.astype(np.float64) - b).max() <= 1e-6
    assert (_bits(a[:, 2]) == _bits(b[:, 2])).all()  # z = u0 in both


@pytest.mark.parametrize("pos,look,fovy,w,h", [((0.5, -1.0, 1.0), (0.5, 0.5, 0.0), 65.0, 256, 256),
                                                ((0.0, 0.0, 35.0), (0.0, 0.0, 0.0), 65.0, 1024, 1024),
                                                ((0.0, 0.0, 3.0), (0.0, 0.0, 0.0), 65.0, 512, 384)])
def test_camera_rays_match_cam_ray(ref, wl, pos, look, fovy, w, h):
    """The workload's pixel-centre rays against the reference's cam_ray on the same camera: same
    origin, t_min and t_max bits; directions within 4 float ulps of 1 (2^-22) per component of
    cam_ray's. The library computes in double and rounds once, so its directions are within half
    an ulp of the exact ones (measured 0.5); cam_ray rounds every float step (measured up to 2.9
    ulps from the exact directions)."""
    got = wl.camera_rays(pos, look, (0.0, 1.0, 0.0), fovy, w, h)
    p, lk = np.asarray(pos, np.float64), np.asarray(look, np.float64)
    d = (lk - p) / np.linalg.norm(lk - p)
    want = np.zeros((w * h, 8), np.float32)
    near = np.zeros(2, np.float32)
    ref.refs_cam_rays(_p(np.asarray(pos, np.float32)), _p(d.astype(np.float32)),
                      _p(np.asarray((0.0, 1.0, 0.0), np.float32)), ctypes.c_float(fovy), w, h, _p(want), _p(near))
    assert (_bits(got[:, 0:3]) == _bits(want[:, 0:3])).all()
    assert (_bits(got[:, 7]) == _bits(want[:, 7])).all()
    # cam_ray's rays keep ray::ray's default t_min (libgi/rt.h:25), the same 1e-4
    assert (_bits(got[:, 3]) == _bits(want[:, 3])).all()
    ulp1 = 2.0 ** -24
    assert np.abs(got[:, 4:7].astype(np.float64) - want[:, 4:7]).max() <= 4 * ulp1
    # the exact directions, in double: normalize(dir + u U + v V)
    U = np.cross(d, (0.0, 1.0, 0.0))
    U /= np.linalg.norm(U)
    V = np.cross(U, d)
    V /= np.linalg.norm(V)
    nh = np.tan(np.pi * fovy * 0.5 / 180)
    x, y = np.tile(np.arange(w), h), np.repeat(np.arange(h), w)
    u, v = ((x + 0.5) / w * 2 - 1) * nh * w / h, ((y + 0.5) / h * 2 - 1) * nh
    exact = d[None, :] + u[:, None] * U[None, :] + v[:, None] * V[None, :]
    exact /= np.linalg.norm(exact, axis=1, keepdims=True)
    assert np.abs(got[:, 4:7] - exact).max() <= 0.5 * ulp1 * (1 + 1e-6)
    assert np.abs(want[:, 4:7] - exact).max() <= 4 * ulp1
    assert abs(float(near[1]) - nh) <= 2 * ulp1 and abs(float(near[0]) - nh * w / h) <= 2 * ulp1
