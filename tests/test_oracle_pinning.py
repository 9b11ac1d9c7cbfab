"""The oracle restatement is pinned to the reference: against golden fixtures made by the
reference's own CPU tracer (tests/golden/make_golden.py), and, where the reference sources are
present, against the reference library itself on further random scenes."""
import numpy as np
import pytest

import cases
from conftest import GOLDEN_CASES, load_golden, same_bits
from make_golden import array_digest, bvh_digest


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_workloads_are_bit_identical(golden_scenes, name):
    g = load_golden(name)
    v, t, rays, _ = golden_scenes[name]
    assert (array_digest(v) == g["vpos_digest"]).all()
    assert (array_digest(t) == g["tris_digest"]).all()
    assert (array_digest(rays) == g["rays_digest"]).all()


@pytest.mark.parametrize("name", GOLDEN_CASES)
@pytest.mark.parametrize("bname,opts", cases.BUILDERS, ids=[b for b, _ in cases.BUILDERS])
def test_oracle_bvh_matches_reference(orc, golden_scenes, name, bname, opts):
    g = load_golden(name)
    v, t, _, _ = golden_scenes[name]
    o = orc.OracleBVH(v, t, **opts)
    assert o.nodes().shape[0] == int(g["nodes_" + bname])
    assert (bvh_digest(o.nodes(), o.index(), o.root) == g["bvh_" + bname]).all()


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_oracle_hits_match_reference(orc, golden_scenes, name):
    g = load_golden(name)
    v, t, rays, any_rays = golden_scenes[name]
    o = orc.OracleBVH(v, t)
    hits, cnt = o.closest(rays, counts=True)
    assert same_bits(hits, g["closest"]).all()
    assert int(cnt[:, 2].max()) <= 24  # the reference's stack holds 25 entries
    occ, _ = o.any(any_rays)
    assert (occ == g["any_occluded"]).all()




@pytest.mark.parametrize("seed,ntri", [(21, 17), (22, 200), (23, 5000), (24, 40000)])
@pytest.mark.parametrize("bname,opts", cases.BUILDERS, ids=[b for b, _ in cases.BUILDERS])
def test_oracle_vs_reference_live(orc, wl, seed, ntri, bname, opts):
    if not orc.ref_available():
        pytest.skip("reference build (oracle/_ref) not present on this host")
    sc = wl.soup(seed, ntri, sigma=0.5 if seed % 2 else 2.0)
    o = orc.OracleBVH(sc.vpos, sc.tris, **opts)
    r = orc.ReferenceBVH(sc.vpos, sc.tris, **opts)
    assert o.root == r.root
    assert (o.nodes() == r.nodes()).all() and (o.index() == r.index()).all()
    if o.depth() <= 23:
        lo, hi = sc.bounds()
        rays = cases.random_rays(seed, 4096, lo, hi)
        assert same_bits(o.closest(rays)[0], r.closest(rays)).all()
        arays = cases.random_rays(seed + 1, 4096, lo, hi, tmax_scale=1.0)
        assert (o.any(arays)[0] == r.any(arays)).all()


def test_oracle_alpha_matches_reference_fixture(orc):
    """The alpha restatement against the reference's alpha-aware tracer (golden_alpha.npz)."""
    g = load_golden("alpha")
    v, t, tc, mat_tex, textures = cases.alpha_scene()
    rays, any_rays = cases.alpha_rays()
    alpha = orc.AlphaSet(tc, mat_tex, textures)
    for key, a in (("vpos", v), ("tris", t), ("tc", tc), ("texels", alpha.texels), ("rays", rays),
                   ("any_rays", any_rays)):
        assert (array_digest(a) == g[key + "_digest"]).all(), key
    o = orc.OracleBVH(v, t)
    o.set_alpha(alpha)
    assert same_bits(o.closest(rays)[0], g["closest"]).all()
    assert (o.any(any_rays)[0] == g["any_occluded"]).all()
    # the textures matter: without alpha some answers change
    o.set_alpha(None)
    assert not same_bits(o.closest(rays)[0], g["closest"]).all()


@pytest.mark.parametrize("seed", [31, 32, 33])
def test_oracle_alpha_vs_reference_live(orc, wl, seed):
    """Random soups with random texture coordinates (wide range, negative values) and random
    alpha textures, against the reference's alpha-aware tracer."""
    if not orc.ref_available():
        pytest.skip("reference build (oracle/_ref) not present on this host")
    g = np.random.default_rng(seed)
    sc = wl.soup(seed, 3000, sigma=0.5)
    nm = 5
    t = sc.tris.copy()
    t[:, 3] = g.integers(0, nm, t.shape[0])
    tc = (g.normal(size=(sc.vpos.shape[0], 2)) * 3.0).astype(np.float32)
    textures = [g.choice(np.float32([0.0, 0.5, 0.51, 1.0]), size=(int(g.integers(1, 9)), int(g.integers(1, 9))))
                for _ in range(3)]
    alpha = orc.AlphaSet(tc, np.array([-1, 0, 1, 2, 1], np.int32), textures)
    o = orc.OracleBVH(sc.vpos, t)
    o.set_alpha(alpha)
    r = orc.ReferenceAlphaBVH(sc.vpos, t, alpha)
    lo, hi = sc.bounds()
    rays = cases.random_rays(seed, 4096, lo, hi)
    assert same_bits(o.closest(rays)[0], r.closest(rays)).all()
    arays = cases.random_rays(seed + 1, 4096, lo, hi, tmax_scale=1.0)
    assert (o.any(arays)[0] == r.any(arays)).all()
