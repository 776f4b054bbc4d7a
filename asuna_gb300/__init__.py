"""asuna_gb300 — GB300-native path-tracer core behind Asuna's scene/plugin API.

The hot path (software BVH traversal + wavefront integrator) is CUDA for
sm_103a in the native library ``_build/libasuna_rt.so`` (C ABI:
include/asuna_rt.h).  This package is the Python host mirror: scene
assembly, cameras, shots, films and render calls.  There is no CPU fallback:
without the native library or a CUDA device the calls raise ``AsunaError``.
"""
from ._abi import AsunaError, lib  # noqa: F401
from .scene import (Context, DeviceScene, Film, JsonScene, SceneBuilder, default_material, default_post,  # noqa: F401
                    default_state,
                    envmap_tables, make_shot, opencv_camera, perspective_camera, set_channels)
