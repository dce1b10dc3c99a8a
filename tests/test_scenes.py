"""Synthetic workload generators: sizes, ranges and determinism."""
import numpy as np

from visionaray_gb300 import scenes


def test_soup_ranges_and_determinism():
    a = scenes.soup(1000, seed=5, offset=0.02)
    b = scenes.soup(1000, seed=5, offset=0.02)
    assert a.tobytes() == b.tobytes()
    assert (a["prim_id"] == np.arange(1000)).all()
    v1 = a["v1"]
    assert v1.min() >= -0.02 and v1.max() <= 1.02
    assert np.abs(a["e1"]).max() <= 0.08 and np.abs(a["e2"]).max() <= 0.08
    assert scenes.soup(1000, seed=6).tobytes() != a.tobytes()


def test_heightfield_layout():
    g = 16
    t = scenes.heightfield(grid=g, seed=1)
    assert len(t) == 2 * g * g
    # cell (0,0): triangle 0 = (P00, P10, P11), triangle 1 = (P00, P11, P01)
    assert np.allclose(t["v1"][0][:2], (0, 0)) and np.allclose(t["e1"][0][:2], (1 / g, 0))
    assert np.allclose(t["e2"][0][:2], (1 / g, 1 / g)) and np.allclose(t["e2"][1][:2], (0, 1 / g))
    # normals point up (+z)
    n = np.cross(t["e1"], t["e2"])
    assert (n[:, 2] > 0).all()
    assert np.abs(t["v1"][:, 2]).max() < 0.1


def test_surface_rays():
    t = scenes.heightfield(grid=32, seed=2)
    c, a = scenes.surface_rays(t, 100, seed=3, ao_per_origin=8, ao_tmax=0.05)
    assert len(c) == 100 and len(a) == 800
    assert np.allclose(np.linalg.norm(c["dir"], axis=1), 1, atol=1e-6)
    assert (a["tmax"] == np.float32(0.05)).all()
    assert (a["ori"].reshape(100, 8, 3) == c["ori"][:, None, :]).all()
    assert (c["dir"][:, 2] > 0).mean() > 0.8   # cosine lobes about upward-facing normals


def test_pinhole_rays():
    r = scenes.pinhole_rays(4, 2)
    assert len(r) == 8
    assert np.allclose(r["ori"], (0.5, 0.5, -1.5))
    assert (r["dir"][:, 2] > 0).all()
    assert np.allclose(np.linalg.norm(r["dir"], axis=1), 1, atol=1e-6)
    # image x grows towards -x in world space (the look_at basis of pinhole_camera)
    assert r["dir"][0, 0] > r["dir"][3, 0]
