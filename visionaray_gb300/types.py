"""numpy views of the C-ABI structs in include/visionaray_gb300/gbrt.h.

The layouts are visionaray's own: basic_triangle<3, float, unsigned>
(math/triangle.h:18-36, 44 bytes), basic_ray<float> (math/ray.h:16-45, 32 bytes),
bvh_node (bvh.h:70-141, 32 bytes) and the (prim_id, t, u, v) part of
hit_record<ray, primitive<unsigned>> (math/intersect.h:151-169).
"""
import numpy as np

TRIANGLE = np.dtype([("geom_id", "<u4"), ("prim_id", "<u4"),
                     ("v1", "<f4", (3,)), ("e1", "<f4", (3,)), ("e2", "<f4", (3,))])
RAY = np.dtype([("ori", "<f4", (3,)), ("dir", "<f4", (3,)),
                ("tmin", "<f4"), ("tmax", "<f4")])
HIT = np.dtype([("prim_id", "<u4"), ("t", "<f4"), ("u", "<f4"), ("v", "<f4")])
BVH_NODE = np.dtype([("bbox_min", "<f4", (3,)), ("bbox_max", "<f4", (3,)),
                     ("first", "<u4"), ("num_prims", "<u2"),
                     ("axis", "u1"), ("sign", "u1")])

# path tracing (gbrt.h): gbrt_material, gbrt_area_light, gbrt_camera, gbrt_pt_params
MATERIAL = np.dtype([("kind", "<u4"), ("color", "<f4", (3,)), ("scale", "<f4"), ("ior", "<f4", (3,)),
                     ("absorption", "<f4", (3,)), ("color2", "<f4", (3,)), ("scale2", "<f4"),
                     ("exponent", "<f4")])
AREA_LIGHT = np.dtype([("geometry", TRIANGLE), ("cl", "<f4", (3,)), ("kl", "<f4")])
LIGHT = np.dtype([("kind", "<u4"), ("cl", "<f4", (3,)), ("kl", "<f4"), ("geometry", TRIANGLE),
                  ("position", "<f4", (3,)), ("attenuation", "<f4", (3,)), ("spot_direction", "<f4", (3,)),
                  ("spot_cutoff", "<f4"), ("spot_exponent", "<f4")])
LIGHT_AREA, LIGHT_POINT, LIGHT_SPOT = 0, 1, 2

# gbrt_environment: the texel pointer (device for the product, host for the oracle),
# texture size, filter and address mode, scale and the column-major light_to_world.
ENVIRONMENT = np.dtype([("texels", "<u8"), ("width", "<u4"), ("height", "<u4"), ("filter", "<u4"),
                        ("address", "<u4"), ("scale", "<f4", (3,)), ("light_to_world", "<f4", (16,))], align=True)
FILTER_NEAREST, FILTER_LINEAR = 0, 1
ADDRESS_WRAP, ADDRESS_MIRROR, ADDRESS_CLAMP = 0, 1, 2


def environment(texels_ptr, width, height, filter=FILTER_LINEAR, address=ADDRESS_CLAMP, scale=(1.0, 1.0, 1.0),
                light_to_world=None):
    """One ENVIRONMENT record; light_to_world is a 4x4 (row, column) matrix, stored
    column-major (identity when None)."""
    e = np.zeros(1, ENVIRONMENT)
    e["texels"], e["width"], e["height"] = texels_ptr, width, height
    e["filter"], e["address"], e["scale"] = filter, address, scale
    m = np.eye(4, dtype=np.float32) if light_to_world is None else np.asarray(light_to_world, np.float32)
    e["light_to_world"] = m.T.reshape(16)
    return e


def lights_of_area_lights(area_lights):
    """AREA_LIGHT records as LIGHT records of kind LIGHT_AREA."""
    a = np.asarray(area_lights, AREA_LIGHT).reshape(-1)
    out = np.zeros(len(a), LIGHT)
    out["kind"] = LIGHT_AREA
    out["geometry"], out["cl"], out["kl"] = a["geometry"], a["cl"], a["kl"]
    return out


CAMERA = np.dtype([("eye", "<f4", (3,)), ("center", "<f4", (3,)), ("up", "<f4", (3,)),
                   ("fovy_degrees", "<f4")])
PT_PARAMS = np.dtype([("width", "<u4"), ("height", "<u4"), ("spp", "<u4"), ("num_bounces", "<u4"),
                      ("epsilon", "<f4"), ("frame_id", "<u4"), ("sfactor", "<f4"), ("dfactor", "<f4"),
                      ("background", "<f4", (4,)), ("ambient", "<f4", (3,)), ("flags", "<u4")])
INSTANCE = np.dtype([("blas", "<u8"), ("transform", "<f4", (12,))])
HIT_INST = np.dtype([("prim_id", "<u4"), ("inst_id", "<u4"), ("t", "<f4"), ("u", "<f4"), ("v", "<f4"),
                     ("geom_id", "<u4"), ("reserved", "<u4", (2,))])
BATCH_LAUNCH = np.dtype([("block", "<u4"), ("tile", "<u4"), ("stack", "<u4"), ("order", "<u4"), ("width", "<u4"),
                         ("sort", "<u4")])
MATTE, EMISSIVE, MIRROR, GLASS, PLASTIC = 0, 1, 2, 3, 4
BATCH_ORDER_ROWS, BATCH_ORDER_BLOCKS = 0, 1
PT_SHADOW_RANGE_FIX = 1
PT_NO_RUSSIAN_ROULETTE = 2
PT_MEGAKERNEL = 4
PT_SORT_QUEUES = 8

NO_HIT = 0xFFFFFFFF
FLT_MAX = float(np.finfo(np.float32).max)

assert TRIANGLE.itemsize == 44 and RAY.itemsize == 32
assert HIT.itemsize == 16 and BVH_NODE.itemsize == 32
assert MATERIAL.itemsize == 64 and AREA_LIGHT.itemsize == 60 and CAMERA.itemsize == 40
assert PT_PARAMS.itemsize == 64 and BATCH_LAUNCH.itemsize == 24
assert INSTANCE.itemsize == 56 and HIT_INST.itemsize == 32
