"""Edge cases of the materials beyond matte, shared by the oracle and GPU tests: a box
whose blobs cycle a plastic with zero reflectances (the lobe choice falls back to
1/2 : 1/2), a plastic with exponent 0 and one with a non-integer exponent (7.5), glass
of index 1 (no bending, no reflection) and of index 2.4 (more total internal
reflection), and a mirror of index 1 without absorption."""

import numpy as np

from visionaray_gb300 import scenes
from visionaray_gb300.types import GLASS, MIRROR, PLASTIC


def edge_material_box(subdiv=6):
    kinds = 6
    tris, mats, lights = scenes.box_scene(n_blobs=2 * kinds, subdiv=subdiv, seed=2)
    per = 20 * subdiv * subdiv
    for b in range(2 * kinds):
        sl = slice(14 + b * per, 14 + (b + 1) * per)
        k = b % kinds
        m = mats[sl]
        m["scale"], m["scale2"] = 1.0, 1.0
        if k == 0:
            m["kind"], m["color"], m["color2"], m["exponent"] = PLASTIC, 0.0, 0.0, 8.0
        elif k == 1:
            m["kind"], m["color"], m["color2"], m["exponent"] = PLASTIC, (0.3, 0.6, 0.2), 0.5, 0.0
        elif k == 2:
            m["kind"], m["color"], m["color2"], m["exponent"] = PLASTIC, (0.6, 0.3, 0.2), 0.3, 7.5
        elif k == 3:
            m["kind"], m["color"], m["color2"], m["ior"] = GLASS, 1.0, 1.0, 1.0
        elif k == 4:
            m["kind"], m["color"], m["color2"], m["ior"] = GLASS, (0.9, 1.0, 0.95), 1.0, 2.4
        else:
            m["kind"], m["color"], m["ior"], m["absorption"] = MIRROR, 0.9, 1.0, 0.0
        mats[sl] = m
    return tris, mats, lights


def env_texels(width=64, height=32, seed=5):
    """A seeded lat-long map (height, width, 4) float32: a sky gradient, noise and a
    bright patch (the sun)."""
    rng = np.random.default_rng(seed)
    v = (np.arange(height, dtype=np.float32) + 0.5) / height
    t = np.zeros((height, width, 4), np.float32)
    t[..., 0] = 0.2 + 0.6 * v[:, None]
    t[..., 1] = 0.3 + 0.4 * v[:, None]
    t[..., 2] = 0.9 - 0.5 * v[:, None]
    t[..., :3] += rng.uniform(0.0, 0.1, size=(height, width, 3)).astype(np.float32)
    t[height // 5: height // 5 + 3, width // 3: width // 3 + 4, :3] = 20.0
    t[..., 3] = 1.0
    return t


# light_to_world transforms: identity, a quarter turn about y (exact inverse) and a
# general rotation with a translation (the translation does not move directions)
ENV_TRANSFORMS = {
    "identity": np.eye(4, dtype=np.float32),
    "quarter_turn": np.array([[0, 0, 1, 0], [0, 1, 0, 0], [-1, 0, 0, 0], [0, 0, 0, 1]], np.float32),
    "rotation": np.array([[0.8, -0.36, 0.48, 2.0], [0.6, 0.48, -0.64, -1.0], [0.0, 0.8, 0.6, 0.5],
                          [0, 0, 0, 1]], np.float32),
}


def open_blob_scene(n_blobs=8, subdiv=8, seed=1):
    """The box scene's blobs without the walls (rays leave the scene), its lights, and a
    camera looking in from outside."""
    tris, mats, lights = scenes.box_scene(n_blobs=n_blobs, subdiv=subdiv, seed=seed)
    cam = scenes.box_camera(eye=(0.5, 0.5, -2.0), center=(0.5, 0.5, 0.5), fovy_degrees=35.0)
    return tris[14:].copy(), mats, lights, cam
