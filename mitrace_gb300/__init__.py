"""GB300-native (sm_103a) drop-in for MiTrace's path-tracing hot path.

The product is ``libmitrace_gb300.so`` (hand-written CUDA kernels behind the C
ABI in ``include/mitrace_gpu.h``).  This package is its Python binding plus the
synthetic scene generators; importing it fails loudly when the library has not
been built.
"""
from . import _abi
from ._abi import MTError
from .scenes import (
    SceneData,
    MeshData,
    MaterialData,
    InstanceData,
    LightData,
    CameraData,
    TextureData,
    PackedScene,
    make_config,
    box_room,
    material_grid,
    large_scene,
    incoherent_rays,
    scene_bounds,
)
from .tracer import Tracer, Stats, brdf_batch, brdf_sample_batch, bvh_build, image_rgb8_device, nrc_encode_device, write_hdr, write_png

__all__ = [
    "MTError",
    "SceneData",
    "MeshData",
    "MaterialData",
    "InstanceData",
    "LightData",
    "CameraData",
    "TextureData",
    "PackedScene",
    "make_config",
    "box_room",
    "material_grid",
    "large_scene",
    "incoherent_rays",
    "scene_bounds",
    "Tracer",
    "Stats",
    "brdf_batch",
    "brdf_sample_batch",
    "bvh_build",
    "nrc_encode_device",
    "image_rgb8_device",
    "write_png",
    "write_hdr",
]
