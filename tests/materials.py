"""Edge cases of the materials beyond matte, shared by the oracle and GPU tests: a box
whose blobs cycle a plastic with zero reflectances (the lobe choice falls back to
1/2 : 1/2), a plastic with exponent 0 and one with a non-integer exponent (7.5), glass
of index 1 (no bending, no reflection) and of index 2.4 (more total internal
reflection), and a mirror of index 1 without absorption."""

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
