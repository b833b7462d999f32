"""seesharp_gb300: SeeSharp's unidirectional PathTracer as a GB300 (sm_103a) wavefront renderer.

The Python classes mirror SeeSharp's scene and integrator API; rendering and ray queries run in
libsst.so (CUDA, C ABI in include/sst.h).
"""
from .images import (BorderHandling, FrameBuffer, MonochromeImage, OutlierReplayCache, Pixel, RgbColor, RgbImage, TextureMono,
                     TextureRgb, mean_rgb, rel_mse, rel_mse_outlier_rejection)
from .integrators import Integrator, PathTracer, autotune, render_batch
from .scene import (ArgumentException, DiffuseEmitter, DiffuseMaterial, EnvironmentMap, GenericMaterial, GlossyEmitter,
                    InvalidOperationException, Matrix4x4, Mesh, PerspectiveCamera, Scene, Triangle)

__all__ = ["BorderHandling", "FrameBuffer", "MonochromeImage", "OutlierReplayCache", "Pixel", "RgbColor", "RgbImage", "TextureMono",
           "TextureRgb", "mean_rgb", "rel_mse", "rel_mse_outlier_rejection", "Integrator", "PathTracer", "autotune", "render_batch", "ArgumentException", "DiffuseEmitter", "DiffuseMaterial", "EnvironmentMap",
           "GenericMaterial", "GlossyEmitter", "InvalidOperationException", "Matrix4x4", "Mesh", "PerspectiveCamera", "Scene",
           "Triangle"]
