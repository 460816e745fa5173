"""GB300-native rendering hot path of go-progressive-raytracer.

Host-side mirror of the reference's Go API (scene, integrators, progressive
renderer) over the C ABI of include/gprt.h, implemented by the CUDA library
built from ../csrc.
"""
from . import _capi as capi  # noqa: F401
from .renderer import (BDPTIntegrator, Context, GpuScene, PassResult, PathTracingIntegrator,  # noqa: F401
                       ProgressiveConfig, ProgressiveRaytracer, RenderStats, TileCompletionResult)
from .scene import (Box, CameraConfig, Cone, Cylinder, Dielectric, Disc, Emissive, Lambertian, Layered,  # noqa: F401
                    ImageTexture, MaterialTable, Mesh, Metal, Mix, NewCheckerboardTexture, NewGradientTexture,
                    NewGroundQuad, NewUVDebugTexture, Quad, SamplingConfig, Scene, Sphere, SpotEmissive,
                    TexturedLambertian, TexturedMetal, Triangle, TriangleMesh)
from . import scenes  # noqa: F401
from .server import RenderServer, ServerEvent, latency_summary  # noqa: F401
