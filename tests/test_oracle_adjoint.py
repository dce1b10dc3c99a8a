"""The oracle's FP64 path-replay adjoint against FP64 central differences of the
oracle's own FP64 forward pass at the same random numbers, on the 4,094-triangle
inverse-rendering box at a generic albedo state (U[0.3, 0.7] per channel: no ties in
the next-event MIS weight's max(throughput)).  This pins the adjoint's mathematics;
the GPU adjoint is compared with this one (tests/test_gpu_full_size.py)."""
import numpy as np

from visionaray_gb300 import scenes
from visionaray_gb300.types import PT_NO_RUSSIAN_ROULETTE, PT_SHADOW_RANGE_FIX


def test_fp64_host_adjoint_equals_fp64_central_differences(oracle):
    tris, mats, lights = scenes.box_scene(n_blobs=204, subdiv=1, seed=1)
    cam = scenes.box_camera()
    params = scenes.pt_params(48, 32, 2, num_bounces=6, frame_id=0, flags=PT_SHADOW_RANGE_FIX | PT_NO_RUSSIAN_ROULETTE)
    tree = oracle.build_sah(tris)
    rng = np.random.default_rng(7)
    albedo = rng.uniform(0.3, 0.7, size=(len(mats), 3)).astype(np.float32)
    emission = np.ascontiguousarray(mats["color"], np.float32)
    adj = rng.normal(size=(32, 48, 4))
    adj[..., 3] = 0.0
    ga, ge, _ = oracle.pathtrace_adjoint(tree, tris, mats, lights, cam, params, albedo, emission, adj, fp64=True)

    def loss(a):
        _, _, img = oracle.pathtrace_adjoint(tree, tris, mats, lights, cam, params, a, emission, np.zeros_like(adj),
                                             fp64=True)
        return float((img * adj).sum())

    nonzero = np.flatnonzero(np.abs(ga).ravel() > 0)
    for k in rng.choice(nonzero, 16, replace=False):
        slot, c = int(k // 3), int(k % 3)
        plus, minus = albedo.copy(), albedo.copy()
        plus[slot, c] += np.float32(1e-3)
        minus[slot, c] -= np.float32(1e-3)
        fd = (loss(plus) - loss(minus)) / float(plus[slot, c] - minus[slot, c])
        # the image is a polynomial in the albedos: only the O(h^2) remainder and FP64
        # rounding separate the two
        assert abs(ga[slot, c] - fd) <= 1e-4 * abs(fd), (slot, c, ga[slot, c], fd)
