"""The FP64 adjoint oracle matches FP64 central finite differences: pins the analytic gradient
formula before it is used to check the GPU adjoint. Richardson extrapolation of the central
differences at h = 1e-4 and h/2 makes the check fourth-order accurate, so it holds tightly even
for near-grazing rays, whose plain central differences carry visible truncation error."""
import numpy as np
import pytest


def _scene(seed):
    g = np.random.default_rng(seed)
    nv, nt, n = 60, 40, 200
    v = g.normal(size=(nv, 3))
    t = np.zeros((nt, 4), np.uint32)
    t[:, :3] = np.stack([g.choice(nv, 3, replace=False) for _ in range(nt)])
    refs = g.integers(0, nt, n).astype(np.uint32)
    # rays from random origins aimed at an interior point of their triangle
    bary = g.dirichlet([2, 2, 2], size=n)
    tri = t[refs, :3]
    target = (bary[:, :1] * v[tri[:, 0]] + bary[:, 1:2] * v[tri[:, 1]] + bary[:, 2:] * v[tri[:, 2]])
    o = target + g.normal(size=(n, 3)) * 3
    d = target - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return v, t, np.concatenate([o, d], axis=1), refs


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_adjoint64_matches_finite_differences(orc, seed):
    v, t, rays, refs = _scene(seed)
    g = np.random.default_rng(seed + 10)
    w = g.normal(size=(refs.size, 3))  # L = sum w . (t, beta, gamma)

    def loss(vv, rr):
        x = orc.fixed_hits64(vv, t, rr, refs)
        return float((w * x).sum())

    gv, gr = orc.adjoint64(v, t, rays, refs, w)

    def richardson(f, x, idx, h=1e-4):
        def central(hh):
            xp, xm = x.copy(), x.copy()
            xp[idx] += hh
            xm[idx] -= hh
            return (f(xp) - f(xm)) / (2 * hh)
        return (4 * central(h / 2) - central(h)) / 3

    for k in g.choice(v.shape[0], 10, replace=False):
        for a in range(3):
            fd = richardson(lambda vv: loss(vv, rays), v, (k, a))
            assert abs(fd - gv[k, a]) <= 1e-6 * max(1.0, abs(fd))
    for r in g.choice(refs.size, 10, replace=False):
        for a in range(6):
            fd = richardson(lambda rr: loss(v, rr), rays, (r, a))
            assert abs(fd - gr[r, a]) <= 1e-6 * max(1.0, abs(fd))
