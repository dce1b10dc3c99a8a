"""Two-level instancing on the GPU against the oracle's brute-force instance query
(pinned to visionaray's index_bvh over index_bvh_inst_t by test_oracle_reference.py)."""
import numpy as np
import pytest

import visionaray_gb300 as vg
from visionaray_gb300.types import NO_HIT

from .instancing import compare_inst, make_instances, make_rays

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scene():
    meshes, inst_mesh, transforms = make_instances()
    blas = [vg.lbvh_builder().build(vg.as_device_bytes(m)) for m in meshes]
    tlas = vg.TLAS([(blas[m], transforms[k]) for k, m in enumerate(inst_mesh)])
    return meshes, inst_mesh, transforms, blas, tlas


def test_closest_and_any_hit_match_oracle(oracle, scene):
    meshes, inst_mesh, transforms, _, tlas = scene
    rays = make_rays()
    d_rays = vg.device_rays(rays)
    trees = [oracle.build_sah(m) for m in meshes]
    insts = [(trees[m], meshes[m], transforms[k]) for k, m in enumerate(inst_mesh)]
    got = vg.hits_inst_to_numpy(tlas.closest_hit(d_rays), len(rays))
    got_any = vg.hits_inst_to_numpy(tlas.any_hit(d_rays), len(rays))
    tlas.ctx.synchronize()
    want = oracle.trace_instances(insts, rays)
    assert (want["prim_id"] != NO_HIT).sum() > len(rays) // 4
    assert compare_inst(got, want) <= len(rays) // 1000
    hit = got["prim_id"] != NO_HIT
    geoms = np.array([meshes[inst_mesh[k]][p]["geom_id"] for k, p in zip(got["inst_id"][hit], got["prim_id"][hit])])
    assert (got["geom_id"][hit] == geoms).all()
    assert ((got_any["prim_id"] != NO_HIT) == hit).all()


def test_empty_and_single_instance(oracle):
    from .instancing import make_rays
    rays = make_rays(512)
    d_rays = vg.device_rays(rays)
    empty = vg.TLAS([])
    h = vg.hits_inst_to_numpy(empty.closest_hit(d_rays), len(rays))
    empty.ctx.synchronize()
    assert (h["prim_id"] == NO_HIT).all() and (h["inst_id"] == NO_HIT).all()
    tri = np.zeros(1, vg.TRIANGLE)
    tri["v1"], tri["e1"], tri["e2"] = (-1.0, -1.0, 0.0), (2.0, 0.0, 0.0), (0.0, 2.0, 0.0)
    one = vg.lbvh_builder().build(vg.as_device_bytes(tri))
    ident = np.array([1, 0, 0, 0, 1, 0, 0, 0, 1, 0.5, 0.0, 0.0], np.float32)
    t = vg.TLAS([(one, ident)])
    got = vg.hits_inst_to_numpy(t.closest_hit(d_rays), len(rays))
    t.ctx.synchronize()
    want = oracle.trace_instances([(oracle.build_sah(tri), tri, ident)], rays)
    assert compare_inst(got, want) == 0


def test_many_and_coincident_instances(oracle):
    """The binned-SAH top level over 300 instances, 40 of them at one transform (their
    centroids in one bin: the median split takes over) and the rest spread out: hits
    equal the oracle's except equal-t ties (the coincident instances tie with each
    other on every ray that meets them)."""
    meshes, inst_mesh, transforms = make_instances(n_inst=260, seed=21)
    same = transforms[0].copy()
    inst_mesh = np.concatenate([inst_mesh, np.zeros(40, np.uint32)])
    transforms = np.concatenate([transforms, np.repeat(same[None, :], 40, axis=0)])
    blas = [vg.lbvh_builder().build(vg.as_device_bytes(m)) for m in meshes]
    tlas = vg.TLAS([(blas[m], transforms[k]) for k, m in enumerate(inst_mesh)])
    rays = make_rays(2048, seed=22)
    d_rays = vg.device_rays(rays)
    got = vg.hits_inst_to_numpy(tlas.closest_hit(d_rays), len(rays))
    got_any = vg.hits_inst_to_numpy(tlas.any_hit(d_rays), len(rays))
    tlas.ctx.synchronize()
    trees = [oracle.build_sah(m) for m in meshes]
    want = oracle.trace_instances([(trees[m], meshes[m], transforms[k]) for k, m in enumerate(inst_mesh)], rays)
    assert (want["prim_id"] != NO_HIT).sum() > len(rays) // 4
    compare_inst(got, want)
    assert ((got_any["prim_id"] != NO_HIT) == (got["prim_id"] != NO_HIT)).all()
