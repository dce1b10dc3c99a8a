"""visionaray's own GPU kernels (oracle/_ref/vsnray_ref_gpu.cubin, device code built
from the reference headers) against the product's kernels on the same GPU, tree, rays
and random numbers.  The reference is compiled with nvcc's default contraction (fused
multiply-adds), as its own build would be, so hits are compared with the parity bar of
the CPU oracle (prim_id except equal-t ties, t/u/v within a few ulp) rather than bit
for bit; the path-traced image within a stated RMSE."""
import numpy as np
import pytest
import torch

import visionaray_gb300 as vg
from oracle import ref_gpu
from visionaray_gb300 import scenes
from visionaray_gb300.types import AREA_LIGHT, NO_HIT

from .parity import ulp_diff

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not ref_gpu.available(), reason="reference cubin not built (no visionaray headers)")]


@pytest.fixture(scope="module")
def ref():
    return ref_gpu.ReferenceGPU(0)


def test_reference_gpu_traversal_agrees(ref):
    tris = scenes.soup(65536, seed=1)
    rays = scenes.pinhole_rays(256, 256)
    d_tris = vg.as_device_bytes(tris)
    bvh = vg.lbvh_builder().build(d_tris)
    tree = ref.tree(d_tris, bvh)
    d_rays = vg.device_rays(rays)
    for any_hit in (False, True):
        ours = vg.hits_to_numpy((vg.any_hit if any_hit else vg.closest_hit)(d_rays, bvh))
        theirs = torch.empty((len(rays), 4), dtype=torch.float32, device="cuda:0")
        ref.trace(tree, d_rays, theirs, any_hit=any_hit)
        torch.cuda.synchronize()
        theirs = vg.hits_to_numpy(theirs)
        hit_o, hit_t = ours["prim_id"] != NO_HIT, theirs["prim_id"] != NO_HIT
        # occlusion agrees for every ray; the reference's fused arithmetic can move a
        # grazing hit across a triangle edge, so allow a few in a million
        assert (hit_o != hit_t).sum() <= max(2, len(rays) // 100000)
        if not any_hit:
            same = (ours["prim_id"] == theirs["prim_id"]) & hit_o
            assert same.sum() >= 0.999 * hit_o.sum()
            assert np.median(ulp_diff(ours["t"][same], theirs["t"][same])) <= 1
            assert np.percentile(ulp_diff(ours["t"][same], theirs["t"][same]), 99.9) <= 64


@pytest.mark.parametrize("exact", [False, True])
@pytest.mark.parametrize("kind", ["soup", "heightfield"])
def test_reference_gpu_lbvh_build_equals_ours(kind, exact):
    """visionaray's own GPU LBVH build (its kernels in lbvh_builder::build's order, CUB's
    stable merge sort) gives the product's tree byte for byte: nodes in the reference's
    cuda_index_bvh layout and the index array, on a random soup (many equal Morton
    codes) and a heightfield, from both reference builds (the bounds and Morton
    arithmetic has no multiply-add to contract)."""
    tris = scenes.soup(65536, seed=3) if kind == "soup" else scenes.heightfield(grid=256, seed=2)
    d_tris = vg.as_device_bytes(tris)
    ref = ref_gpu.ReferenceGPU(0, exact=exact)
    b = ref.lbvh_buffers(len(tris))
    for name in ("prim_bounds", "centroids", "prim_refs", "inner", "leaves", "nodes", "prims", "indices"):
        b[name].fill_(0xA5)   # the build must not depend on what the buffers held
    nodes_r, idx_r = ref.lbvh_build(d_tris, b)
    bvh = vg.lbvh_builder().build(d_tris)
    nodes_o, idx_o = bvh.export_bvh2()
    torch.cuda.synchronize()
    first = nodes_r.cpu().numpy()   # a copy: the next build reuses the buffers
    assert np.array_equal(first, np.ascontiguousarray(nodes_o).view(np.uint8))
    assert np.array_equal(idx_r.cpu().numpy(), np.ascontiguousarray(idx_o).view(np.uint8))
    # a second build into the same buffers gives the same tree
    nodes_2, _ = ref.lbvh_build(d_tris, b)
    torch.cuda.synchronize()
    assert np.array_equal(nodes_2.cpu().numpy(), first)


def render_pair(exact, tris, mats, lights, cam, params):
    d_tris = vg.as_device_bytes(tris)
    bvh = vg.lbvh_builder().build(d_tris)
    ours = vg.pathtrace_frame(vg.PTScene(bvh, mats, lights), cam, params)
    ref = ref_gpu.ReferenceGPU(0, exact=exact)
    scene = ref.pt_scene(ref.tree(d_tris, bvh), mats, lights)
    theirs = torch.zeros_like(ours)
    ref.pathtrace(scene, cam, params, theirs)
    torch.cuda.synchronize()
    a = ours.cpu().numpy()[..., :3].astype(np.float64)
    b = theirs.cpu().numpy()[..., :3].astype(np.float64)
    d = np.abs(a - b).max(axis=2)
    return {"exact_pixels": float((d == 0).mean()), "close_pixels": float((d <= 1e-4 * max(b.max(), 1e-30)).mean()),
            "rmse": float(np.sqrt(((a - b) ** 2).mean())), "mean": (float(a.mean()), float(b.mean()))}


@pytest.mark.skipif(not ref_gpu.available(exact=True), reason="exact reference cubin not built")
def test_reference_gpu_pathtracer_open_scene():
    """An open soup under ambient light: paths end in the sky after a few diffuse bounces,
    so a last-bit difference in a direction rarely changes a path.  The reference's
    device build normalises with rsqrtf and takes float cos/sin (the product: 1/sqrtf,
    cos/sin in double), so pixels agree to rounding, not bit for bit."""
    tris = scenes.soup(20000, seed=4, offset=0.5 / 20000 ** (1 / 3))
    mats = np.zeros(1, vg.types.MATERIAL)
    mats["kind"], mats["color"], mats["scale"] = 0, (0.7, 0.6, 0.5), 1.0
    cam = scenes.box_camera(eye=(0.5, 0.5, -1.2), center=(0.5, 0.5, 0.5), fovy_degrees=50.0)
    params = scenes.pt_params(96, 64, 4, num_bounces=3, frame_id=3, ambient=(1.0, 1.0, 1.0))
    s = render_pair(True, tris, mats, np.zeros(0, AREA_LIGHT), cam, params)
    print(s)
    # the device build draws the hemisphere sample's two numbers in the other order
    # than the CPU build the product follows: per pixel the renders are different
    # estimates of one image
    assert abs(s["mean"][0] - s["mean"][1]) <= 0.02 * s["mean"][1], s
    # ...and the oracle with the device build's draw order reproduces the device build
    from oracle import Oracle
    orc = Oracle()
    ref = ref_gpu.ReferenceGPU(0, exact=True)
    d_tris = vg.as_device_bytes(tris)
    bvh = vg.lbvh_builder().build(d_tris)
    theirs = torch.zeros((64, 96, 4), dtype=torch.float32, device="cuda:0")
    ref.pathtrace(ref.pt_scene(ref.tree(d_tris, bvh), mats, np.zeros(0, AREA_LIGHT)), cam, params, theirs)
    torch.cuda.synchronize()
    img, _ = orc.pathtrace(orc.build_sah(tris), tris, mats, np.zeros(0, AREA_LIGHT), cam, params,
                           mode=Oracle.PT_FLOAT | Oracle.PT_DRAWS_IN_ORDER)
    b = theirs.cpu().numpy()[..., :3].astype(np.float64)
    d = np.abs(img[..., :3] - b).max(axis=2)
    close = float((d <= 1e-4 * b.max()).mean())
    print("device build vs oracle (draws in order):", close, float(np.sqrt((d ** 2).mean())))
    assert close >= 0.98, close


@pytest.mark.skipif(not ref_gpu.available(exact=True), reason="exact reference cubin not built")
def test_reference_gpu_pathtracer_closed_box():
    """The closed box (area light, or only the emissive quad): light arrives along rare,
    long paths, and the reference's shadow-ray range puts each light sample at the ray's
    tmax, so rounding decides most next-event samples; the two renders are nearly
    independent estimates and agree in the mean only.  8 spp at 192 x 128."""
    tris, mats, lights = scenes.box_scene(n_blobs=8, subdiv=8, seed=1)
    cam = scenes.box_camera()
    params = scenes.pt_params(192, 128, 8, num_bounces=8, frame_id=11)
    for exact in (True, False):
        s = render_pair(exact, tris, mats, lights, cam, params)
        print(exact, s)
        assert np.isclose(s["mean"][0], s["mean"][1], rtol=0.1), s


def material_soup(n=20000, seed=4):
    """A soup whose triangles cycle matte, mirror, glass and plastic slots."""
    from visionaray_gb300.types import GLASS, MATERIAL, MIRROR, PLASTIC
    tris = scenes.soup(n, seed=seed, offset=0.5 / n ** (1 / 3))
    tris["geom_id"] = tris["prim_id"] % 4
    mats = np.zeros(4, MATERIAL)
    mats["kind"] = (0, MIRROR, GLASS, PLASTIC)
    mats["color"] = ((0.7, 0.6, 0.5), (0.9, 0.9, 0.8), (1.0, 1.0, 1.0), (0.2, 0.5, 0.7))
    mats["scale"] = 1.0
    mats["ior"] = ((1.0, 1.0, 1.0), (0.27, 0.42, 1.35), (1.5, 1.5, 1.5), (1.0, 1.0, 1.0))
    mats["absorption"][1] = (3.4, 2.3, 1.8)
    mats["color2"][2], mats["scale2"][2] = (1.0, 1.0, 1.0), 1.0
    mats["color2"][3], mats["scale2"][3], mats["exponent"][3] = (0.5, 0.5, 0.5), 1.0, 24.0
    return tris, mats


@pytest.mark.skipif(not ref_gpu.available(exact=True), reason="exact reference cubin not built")
def test_reference_gpu_materials_and_point_light_open_scene():
    """Mirror, glass and plastic slots and a point light through the reference's
    generic_material / generic_light instantiation on the GPU: the device build (first
    hemisphere draw first, rsqrtf normalisation) against the oracle with the device
    build's draw order; and the product's mean against it."""
    from oracle import Oracle
    from visionaray_gb300.types import LIGHT, LIGHT_POINT
    tris, mats = material_soup()
    lights = np.zeros(1, LIGHT)
    lights["kind"], lights["cl"], lights["kl"] = LIGHT_POINT, (1.0, 0.9, 0.8), 0.5
    lights["position"], lights["attenuation"] = (0.5, 1.6, -0.4), (1.0, 0.0, 0.0)
    cam = scenes.box_camera(eye=(0.5, 0.5, -1.2), center=(0.5, 0.5, 0.5), fovy_degrees=50.0)
    params = scenes.pt_params(96, 64, 4, num_bounces=4, frame_id=3, ambient=(0.5, 0.6, 0.7))
    s = render_pair(True, tris, mats, lights, cam, params)
    print(s)
    assert abs(s["mean"][0] - s["mean"][1]) <= 0.03 * s["mean"][1], s
    orc = Oracle()
    ref = ref_gpu.ReferenceGPU(0, exact=True)
    d_tris = vg.as_device_bytes(tris)
    bvh = vg.lbvh_builder().build(d_tris)
    theirs = torch.zeros((64, 96, 4), dtype=torch.float32, device="cuda:0")
    rscene = ref.pt_scene(ref.tree(d_tris, bvh), mats, lights)
    assert rscene["ext"]
    ref.pathtrace(rscene, cam, params, theirs)
    torch.cuda.synchronize()
    img, _ = orc.pathtrace(orc.build_sah(tris), tris, mats, lights, cam, params,
                           mode=Oracle.PT_FLOAT | Oracle.PT_DRAWS_IN_ORDER)
    b = theirs.cpu().numpy()[..., :3].astype(np.float64)
    d = np.abs(img[..., :3] - b).max(axis=2)
    close = float((d <= 1e-4 * b.max()).mean())
    print("device build vs oracle (draws in order):", close, float(np.sqrt((d ** 2).mean())))
    assert close >= 0.9, close


@pytest.mark.skipif(not ref_gpu.available(exact=True), reason="exact reference cubin not built")
def test_reference_gpu_glossy_box_mixed_lights():
    """The glossy box lit by area, point and spot lights: means agree (closed box, see
    test_reference_gpu_pathtracer_closed_box)."""
    tris, mats, area = scenes.glossy_box_scene(n_blobs=10, subdiv=8, seed=1)
    lights = scenes.mixed_lights(area)
    cam = scenes.box_camera()
    params = scenes.pt_params(192, 128, 8, num_bounces=8, frame_id=12)
    for exact in (True, False):
        s = render_pair(exact, tris, mats, lights, cam, params)
        print(exact, s)
        assert np.isclose(s["mean"][0], s["mean"][1], rtol=0.1), s
