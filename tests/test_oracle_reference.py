"""Direct oracle-vs-reference comparisons on extra inputs, where visionaray's own CPU
code was compiled (oracle/_ref); skipped elsewhere (the GPU host has no sources)."""
import numpy as np
import pytest

from oracle import Reference
from visionaray_gb300 import scenes

pytestmark = pytest.mark.skipif(not Reference.available(), reason="visionaray sources not built here")


@pytest.fixture(scope="module")
def ref():
    return Reference()


@pytest.mark.parametrize("n,seed,offset", [(1, 3, 0.02), (2, 4, 0.02), (3, 5, 0.3), (5, 6, 0.0),
                                          (1000, 7, 0.05), (20000, 8, 0.01)])
def test_builders_and_traversal_match(oracle, ref, n, seed, offset):
    tris = scenes.soup(n, seed=seed, offset=offset)
    rays = scenes.pinhole_rays(64, 48, eye=(0.5, 0.5, -1.0), fovy_degrees=60.0)
    for build in ("build_sah", "build_lbvh_cpu"):
        t_o = getattr(oracle, build)(tris)
        h_r = getattr(ref, build)(tris)
        t_r = h_r.tree()
        assert np.array_equal(t_o.nodes, t_r.nodes) and np.array_equal(t_o.indices, t_r.indices), build
        for any_hit in (False, True):
            a, ca = oracle.trace(t_o, tris, rays, any_hit=any_hit, counters=True)
            b, cb = h_r.trace(rays, any_hit=any_hit, counters=True)
            assert np.array_equal(a, b) and np.array_equal(ca, cb), (build, any_hit)


def test_duplicate_centroids(oracle, ref):
    # all triangles share one centroid: SAH refuses to split (size[axis] <= 0), the
    # Karras tree orders equal codes by index
    base = scenes.soup(1, seed=1, offset=0.02)
    tris = np.repeat(base, 50)
    tris["prim_id"] = np.arange(50)
    t_o = oracle.build_sah(tris)
    t_r = ref.build_sah(tris).tree()
    assert np.array_equal(t_o.nodes, t_r.nodes)
    ids, codes = ref.lbvh_sorted_refs(tris)
    assert np.array_equal(oracle.morton_codes(tris)[ids], codes)
    l1, r1 = oracle.karras_children(codes)
    l2, r2 = ref.karras_children(codes)
    assert np.array_equal(l1, l2) and np.array_equal(r1, r2)


def test_karras_children_random_codes(oracle, ref):
    rng = np.random.default_rng(0)
    for n in (2, 3, 17, 1000, 5000):
        codes = np.sort(rng.integers(0, 1 << 12, n).astype(np.uint32))   # many equal codes
        l1, r1 = oracle.karras_children(codes)
        l2, r2 = ref.karras_children(codes)
        assert np.array_equal(l1, l2) and np.array_equal(r1, r2), n


@pytest.mark.parametrize("max_leaf", [1, 4])
def test_refit_matches_reference(oracle, ref, max_leaf):
    """The oracle's refit restatement equals visionaray's bvh_refitter on its own SAH
    tree after the triangles move."""
    tris = scenes.soup(3000, seed=21)
    moved = tris.copy()
    rng = np.random.default_rng(4)
    moved["v1"] += rng.uniform(-0.05, 0.05, size=(len(tris), 3)).astype(np.float32)
    moved["e1"] *= np.float32(1.3)
    h = ref.build_sah(tris, max_leaf=max_leaf)
    before = h.tree()
    h.refit(moved)
    after = h.tree()
    mine = oracle.refit(before, moved)
    assert mine.nodes.tobytes() == after.nodes.tobytes()
    assert np.array_equal(mine.indices, after.indices)


def test_instances_match_reference(oracle, ref):
    """The oracle's two-level query (inverse, transform_ray, per-instance closest hit,
    is_closer) equals visionaray's index_bvh over index_bvh_inst_t."""
    from .instancing import compare_inst, make_instances, make_rays
    meshes, inst_mesh, transforms = make_instances()
    rays = make_rays()
    trees = [oracle.build_sah(m) for m in meshes]
    insts = [(trees[m], meshes[m], transforms[k]) for k, m in enumerate(inst_mesh)]
    for any_hit in (False, True):
        want = ref.trace_instances(meshes, inst_mesh, transforms, rays, any_hit=any_hit)
        got = oracle.trace_instances(insts, rays, any_hit=any_hit)
        assert (want["prim_id"] != 0xFFFFFFFF).sum() > len(rays) // 4
        if any_hit:
            assert ((want["prim_id"] == 0xFFFFFFFF) == (got["prim_id"] == 0xFFFFFFFF)).all()
        else:
            assert compare_inst(got, want) <= len(rays) // 1000
