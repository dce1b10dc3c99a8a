"""The oracle restatement against golden vectors generated from visionaray's own CPU
code (tests/golden/make_golden.py).  Runs on any host: the scenes are bit-identical
on x86-64 and AArch64."""
import hashlib

import numpy as np
import pytest

from visionaray_gb300 import scenes


def digest(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def check_tree(oracle, tree, rec):
    assert len(tree.nodes) == rec["num_nodes"]
    assert len(tree.indices) == rec["num_indices"]
    assert tree.depth == rec["depth"]
    assert digest(tree.nodes, tree.indices) == rec["sha256"]
    assert oracle.sah_cost(tree) == pytest.approx(rec["sah_cost"], rel=0, abs=0)


def check_trace(oracle, tree, tris, rays, any_hit, rec, sample, stride):
    hits, cnt = oracle.trace(tree, tris, rays, any_hit=any_hit, counters=True)
    assert int(cnt[0]) == rec["box_tests"] and int(cnt[1]) == rec["tri_tests"]
    assert int((hits["prim_id"] != 0xFFFFFFFF).sum()) == rec["num_hits"]
    assert np.array_equal(hits[::stride], sample)
    assert digest(hits) == rec["sha256"]


@pytest.fixture(scope="module")
def soup(golden):
    meta, _ = golden
    s = meta["soup"]
    tris = scenes.soup(s["scene"]["n"], seed=s["scene"]["seed"], offset=s["scene"]["offset"])
    rays = scenes.pinhole_rays(1024, 1024)
    return s, tris, rays


def test_soup_inputs_are_the_golden_inputs(soup):
    s, tris, rays = soup
    assert digest(tris) == s["triangles_sha256"]
    assert digest(rays) == s["rays_sha256"]


def test_soup_sah_tree_and_traversal(oracle, soup, golden):
    s, tris, rays = soup
    _, samples = golden
    stride = golden[0]["sample_stride"]
    tree = oracle.build_sah(tris)
    check_tree(oracle, tree, s["sah"])
    check_trace(oracle, tree, tris, rays, False, s["sah_closest"], samples["soup_sah_closest"], stride)
    check_trace(oracle, tree, tris, rays, True, s["sah_any"], samples["soup_sah_any"], stride)


def test_soup_cpu_lbvh_tree_and_traversal(oracle, soup, golden):
    s, tris, rays = soup
    _, samples = golden
    tree = oracle.build_lbvh_cpu(tris)
    check_tree(oracle, tree, s["lbvh_cpu"])
    check_trace(oracle, tree, tris, rays, False, s["lbvh_cpu_closest"], samples["soup_lbvh_closest"],
                golden[0]["sample_stride"])


def test_soup_morton_and_karras(oracle, soup, golden):
    s, tris, _ = soup
    _, samples = golden
    codes = oracle.morton_codes(tris)
    ids = np.argsort(codes, kind="stable").astype(np.int32)
    sorted_codes = codes[ids]
    assert digest(ids, sorted_codes) == s["morton_sorted_sha256"]
    left, right = oracle.karras_children(sorted_codes)
    assert digest(left, right) == s["karras_children_sha256"]


def test_heightfield_case(oracle, golden):
    meta, samples = golden
    h = meta["heightfield"]
    sc, rc = h["scene"], h["rays"]
    tris = scenes.heightfield(grid=sc["grid"], seed=sc["seed"], base_amplitude=sc["base_amplitude"],
                              base_frequency=sc["base_frequency"], octaves=sc["octaves"])
    closest, ao = scenes.surface_rays(tris, rc["origins"], seed=rc["seed"], offset=rc["offset"],
                                      ao_per_origin=rc["ao_per_origin"], ao_tmax=rc["ao_tmax"])
    assert digest(tris) == h["triangles_sha256"]
    assert digest(closest) == h["closest_rays_sha256"] and digest(ao) == h["ao_rays_sha256"]
    tree = oracle.build_sah(tris)
    check_tree(oracle, tree, h["sah"])
    stride = meta["sample_stride"]
    check_trace(oracle, tree, tris, closest, False, h["sah_closest"], samples["hf_sah_closest"], stride)
    check_trace(oracle, tree, tris, ao, True, h["sah_ao_any"], samples["hf_sah_ao_any"], stride)
    codes = oracle.morton_codes(tris)
    ids = np.argsort(codes, kind="stable").astype(np.int32)
    assert digest(ids, codes[ids]) == h["morton_sorted_sha256"]
    left, right = oracle.karras_children(codes[ids])
    assert digest(left, right) == h["karras_children_sha256"]
