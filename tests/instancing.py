"""Shared inputs of the instancing tests: two soups, instances with rotations, non-
uniform scales and translations (visionaray mat4x3 column layout), rays through the
instanced scene."""
import numpy as np

from visionaray_gb300 import scenes
from visionaray_gb300.types import FLT_MAX, RAY


def rotation(rng):
    q, r = np.linalg.qr(rng.normal(size=(3, 3)))
    q = q * np.sign(np.diag(r))
    if np.linalg.det(q) < 0:
        q[:, 0] = -q[:, 0]
    return q


def make_instances(n_inst=24, seed=11):
    rng = np.random.default_rng(seed)
    meshes = [scenes.soup(3000, seed=41, offset=0.03), scenes.soup(1200, seed=42, offset=0.05)]
    inst_mesh, transforms = [], []
    for k in range(n_inst):
        lin = rotation(rng) @ np.diag(rng.uniform(0.5, 1.5, size=3))
        t = rng.uniform(-2.0, 2.0, size=3)
        # mat4x3 columns c0..c2 with row i of the map = column i
        cols = [lin[0, :], lin[1, :], lin[2, :], t]
        transforms.append(np.concatenate(cols).astype(np.float32))
        inst_mesh.append(k % len(meshes))
    return meshes, np.array(inst_mesh, np.uint32), np.array(transforms, np.float32)


def make_rays(n=4096, seed=12):
    rng = np.random.default_rng(seed)
    rays = np.zeros(n, RAY)
    ori = rng.normal(size=(n, 3))
    ori = 6.0 * ori / np.linalg.norm(ori, axis=1, keepdims=True)
    tgt = rng.uniform(-2.5, 2.5, size=(n, 3))
    d = tgt - ori
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays["ori"], rays["dir"] = ori.astype(np.float32), d.astype(np.float32)
    rays["tmin"], rays["tmax"] = 0.0, FLT_MAX
    return rays


def compare_inst(got, ref, max_t_ulp=2):
    """prim_id / inst_id equal except equal-t ties (t within max_t_ulp); where equal,
    t, u, v bit for bit.  Returns the number of ties."""
    from visionaray_gb300.types import NO_HIT

    from .parity import ulp_diff
    same = (got["prim_id"] == ref["prim_id"]) & (got["inst_id"] == ref["inst_id"])
    assert ((got["prim_id"] == NO_HIT) == (ref["prim_id"] == NO_HIT)).all(), "hit/miss disagreement"
    hit = same & (ref["prim_id"] != NO_HIT)
    for f in ("t", "u", "v"):
        assert (got[f][hit].view(np.uint32) == ref[f][hit].view(np.uint32)).all(), f
    ties = ~same
    assert (ulp_diff(got["t"][ties], ref["t"][ties]) <= max_t_ulp).all(), "different hits at different t"
    return int(ties.sum())
