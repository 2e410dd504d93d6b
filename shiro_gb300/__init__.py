"""shiro_gb300 - GB300-native path-tracing backend for Shiro.

The product is the native library ``libshiro_gpu.so`` (hand-written sm_103a
CUDA kernels behind the C ABI of include/shiro_gpu.h).  This package holds its
Python mirror of the reference's backend interface (``GpuBackend``), the
ctypes ABI structs (``abi``), seeded workloads (``scenes``) and the torch
autograd binding of the differentiable form (``autograd``).
"""
from .abi import (Camera, DistantLight, DomeLight, FrameBuffer, Material, Mesh, RenderSettings, Scene,  # noqa: F401
                  lambert, standard_surface, usd_preview_surface)
from .backend import GpuBackend, RenderRequest, ShiroGpuError, load_library  # noqa: F401
