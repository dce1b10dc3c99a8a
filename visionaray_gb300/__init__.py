"""GB300-native (sm_103a) ray-tracing hot path of visionaray: GPU LBVH build and
closest_hit / any_hit traversal behind the C ABI of include/visionaray_gb300/gbrt.h.

The Python layer is a thin host-side mirror of the reference's interface
(runtime.py); all work runs in the CUDA kernels of libgbrt.so.
"""
from .types import (AREA_LIGHT, BATCH_LAUNCH, BVH_NODE, CAMERA, FLT_MAX, HIT, MATERIAL,  # noqa: F401
                    NO_HIT, PT_PARAMS, PT_SHADOW_RANGE_FIX, RAY, TRIANGLE)
from .runtime import (TLAS, Batch, Context, GbrtError, IndexBVH, PTScene, any_hit, closest_hit,  # noqa: F401
                      default_context, device_rays, as_device_bytes, hits_inst_to_numpy, hits_to_numpy,
                      lbvh_builder, load_library, pathtrace_backward, pathtrace_forward, ploc_builder,
                      pathtrace_frame, pinhole_camera_basis)
