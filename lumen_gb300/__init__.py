"""lumen_gb300: GB300-native BVH construction, ray traversal and MIS path tracing behind a C ABI.

The compute path is liblgb.so (CUDA, sm_103a), built in-tree by `lumen_gb300.build.build_library()`.
Python here only stages host arrays and forwards device pointers to the C ABI (include/lgb.h).
"""
from . import abi  # noqa: F401
from .scene import Context, GpuScene, SceneArrays, camera_lookat, path_params  # noqa: F401
