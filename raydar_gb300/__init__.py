"""raydar_gb300: the GB300 (sm_103a) CUDA backend for Raydar's path-tracing hot path.

The product is libraydar_cuda.so (C ABI: include/raydar_cuda.h).  This
package holds its build recipe, a ctypes binding, Raydar's scene model and
`.rscn` format, the seeded scene generator and `CudaRenderer`, the
reference's `trait Renderer` over the C ABI.
"""
from .renderer import CudaRenderer, Profiler, RendererConfig  # noqa: F401
from .scene import Camera, Material, Object, Scene, World, default_scene  # noqa: F401
