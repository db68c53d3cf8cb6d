"""GB300-native (sm_103a) implementation of the per-frame raster pipeline of the Rust software
rasterizer NiklasJonsson/rusterizer.

The compute path is CUDA behind the C ABI in include/rast.h (librast.so, built in-tree by
rusterizer_gb300/build.py); this package is the host-side mirror of the reference's render API
(Renderer, Uniforms, Texture, meshes and matrix helpers) plus the batched and serving front
ends. There is no CPU fallback: without the shared library every render call raises.
"""
from . import math, mesh, scenes  # noqa: F401
from ._lib import (FS_COLOR, FS_DEBUG, FS_TEXTURE, VS_MVP, RastError,  # noqa: F401
                   LIB_PATH, load)
from .renderer import Mesh, Renderer, Texture, UniformBlock, Uniforms, render_scene  # noqa: F401
