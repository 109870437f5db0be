"""syfrack_gb300: SyFrack's distance-estimator hot path on GB300 (sm_103a).

The compute lives in libsyfrack_gpu.so (C ABI: include/syfrack_gpu.h); this
package is its ctypes binding with the reference's Rust API names.
"""
from . import abi, ron
from .graph import Graph, Kind, Link, Node
from .render import (Batch, Canvas, CompiledGraph, DeSample, ExportSession, GpuContext, PlanarFractal, PreviewSession,
                     RenderOutput, Renderer, RenderSession, deep_zoom, escape2d)
from .serve import ServeResult, Server
from .scene import AreaLight, Camera, Finish, Material, ProjectorLight, RenderConfig, Scene, SurfaceVariation, TubeLight
from ._lib import SyfrackError

__all__ = ["abi", "ron", "Batch", "Graph", "Kind", "Link", "Node", "Canvas", "CompiledGraph", "DeSample", "ExportSession",
           "GpuContext", "PreviewSession",
           "PlanarFractal", "RenderOutput", "Renderer", "RenderSession", "ServeResult", "Server", "deep_zoom", "escape2d", "AreaLight",
           "Camera", "Finish", "Material", "RenderConfig", "Scene", "SurfaceVariation", "SyfrackError"]
