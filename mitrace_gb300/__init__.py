"""GB300-native (sm_103a) drop-in for MiTrace's path-tracing hot path.

The product is ``libmitrace_gb300.so`` (hand-written CUDA kernels behind the C
ABI in ``include/mitrace_gpu.h``).  This package is its Python binding plus the
synthetic scene generators.  The scene generators and boundary structs load no
library; the first use of anything that calls the library (``Tracer``,
``MTError``, the batch entry points) imports ``_abi``, which raises when the
library has not been built: there is no fallback.
"""
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

_LIBRARY_NAMES = {
    "MTError": "_abi",
    "Tracer": "tracer",
    "Stats": "tracer",
    "brdf_batch": "tracer",
    "brdf_sample_batch": "tracer",
    "bvh_build": "tracer",
    "image_rgb8_device": "tracer",
    "nrc_encode_device": "tracer",
    "write_hdr": "tracer",
    "write_png": "tracer",
}


def __getattr__(name):
    import importlib

    if name in ("_abi", "tracer", "gltf"):
        return importlib.import_module(f".{name}", __name__)
    mod = _LIBRARY_NAMES.get(name)
    if mod is None:
        raise AttributeError(f"module 'mitrace_gb300' has no attribute {name!r}")
    value = getattr(importlib.import_module(f".{mod}", __name__), name)
    globals()[name] = value
    return value


__all__ = [
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
    *_LIBRARY_NAMES,
]
