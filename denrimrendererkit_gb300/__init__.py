"""GB300 (sm_103a) backend for DenrimRendererKit's progressive path tracer.

The compute path is the in-tree C-ABI library `_lib/libdenrim_cuda.so`
(include/denrim_cuda.h); this package is the host-side mirror of the
reference's Swift API (scene description, scene compile, render session).
"""
from .library import DenrimError, device_count, load  # noqa: F401
from .renderer import DenrimRenderer, RenderOutput, RenderQuality, RenderSession, RenderSettings  # noqa: F401
from .scene import (AccelerationBuild, Camera, Environment, Material, Mesh, QuadLight, RenderScene,  # noqa: F401
                    SceneBounds, Texture2D, Transform, compile_scene, icosphere)

__all__ = [
    "DenrimError", "DenrimRenderer", "RenderOutput", "RenderQuality", "RenderSession", "RenderSettings",
    "AccelerationBuild", "Camera", "Environment", "Material", "Mesh", "QuadLight", "RenderScene", "SceneBounds",
    "Texture2D", "Transform",
    "compile_scene", "icosphere", "device_count", "load",
]
