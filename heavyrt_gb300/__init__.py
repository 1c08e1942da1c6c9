"""GB300 ray-query engine: LBVH build and nearest/any-hit BVH traversal on one
GPU, behind a mirror of HeavyRT's ISceneObject interface.

The compute path is the native library built from heavyrt_gb300/csrc
(libhrt.so, sm_103a); this package only binds it.
"""
from .engine import (  # noqa: F401
    BUILD_HIGH,
    BUILD_LOW,
    BUILD_MEDIUM,
    BUILD_REFIT,
    HIT_DTYPE,
    NODE_DTYPE,
    Context,
    CreateSceneRT,
    DeleteSceneRT,
    Frame,
    HrtError,
    PinnedBuffer,
    SceneRT,
    rtao_qmc_tile,
)

__all__ = [
    "BUILD_HIGH", "BUILD_LOW", "BUILD_MEDIUM", "BUILD_REFIT", "HIT_DTYPE", "NODE_DTYPE", "Context", "CreateSceneRT",
    "DeleteSceneRT", "Frame", "HrtError", "PinnedBuffer", "SceneRT", "rtao_qmc_tile",
]
