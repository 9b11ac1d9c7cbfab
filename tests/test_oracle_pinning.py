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
