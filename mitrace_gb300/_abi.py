"""ctypes mirror of ``include/mitrace_gpu.h`` and the loader of the in-tree
``libmitrace_gb300.so``.

There is no fallback: if the shared library is missing or fails to load, the
import of this module raises, so nothing can silently run without the CUDA
kernels.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

from ._types import *  # noqa: F401,F403  (the header's types and constants)
from ._types import (mt_bvh_node, mt_config, mt_grad_buffers, mt_nrc_config, mt_nrc_stats, mt_profile,
                     mt_scene_desc, mt_stats, STATUS_NAMES, MT_OK)

LIB_PATH = Path(__file__).resolve().parent / "libmitrace_gb300.so"

# Every entry point declared in include/mitrace_gpu.h: (name, restype, argtypes).
_VP = C.c_void_p
PROTOTYPES = [
    ("mt_config_defaults", None, [C.POINTER(mt_config)]),
    ("mt_create", C.c_int, [C.POINTER(mt_scene_desc), C.POINTER(mt_config), C.POINTER(_VP)]),
    ("mt_destroy", None, [_VP]),
    ("mt_release_cached_memory", None, []),
    ("mt_start", C.c_int, [_VP]),
    ("mt_wait", C.c_int, [_VP, _VP]),
    ("mt_kill", C.c_int, [_VP]),
    ("mt_get_stats", C.c_int, [_VP, C.POINTER(mt_stats)]),
    ("mt_is_done", C.c_int, [_VP]),
    ("mt_set_seed", C.c_int, [_VP, C.c_uint64]),
    ("mt_render_device", C.c_int, [_VP, _VP, _VP]),
    ("mt_render_rows_device", C.c_int, [_VP, C.c_uint32, C.c_uint32, _VP, _VP]),
    ("mt_render_rows_noalloc", C.c_int, [_VP, C.c_uint32, C.c_uint32, _VP, _VP]),
    ("mt_render_grad", C.c_int, [_VP, C.POINTER(mt_grad_buffers), _VP]),
    ("mt_update_materials", C.c_int, [_VP, _VP, C.c_uint32]),
    ("mt_update_lights", C.c_int, [_VP, _VP, C.c_uint32]),
    ("mt_update_texture", C.c_int, [_VP, C.c_uint32, _VP]),
    ("mt_nrc_config_defaults", None, [C.POINTER(mt_nrc_config)]),
    ("mt_nrc_enable", C.c_int, [_VP, C.POINTER(mt_nrc_config)]),
    ("mt_nrc_frame", C.c_int, [_VP, _VP, C.c_uint32, _VP]),
    ("mt_nrc_get_stats", C.c_int, [_VP, C.POINTER(mt_nrc_stats)]),
    ("mt_nrc_get_params", C.c_int, [_VP, _VP]),
    ("mt_nrc_set_params", C.c_int, [_VP, _VP]),
    ("mt_nrc_infer", C.c_int, [_VP, _VP, C.c_uint32, _VP, _VP]),
    ("mt_nrc_train_step", C.c_int, [_VP, _VP, _VP, C.c_uint32, _VP, _VP, _VP]),
    ("mt_nrc_encode", C.c_int, [_VP, C.c_uint32, _VP, _VP]),
    ("mt_trace_rays", C.c_int, [_VP, _VP, C.c_uint64, _VP, C.c_int]),
    ("mt_trace_rays_device", C.c_int, [_VP, _VP, C.c_uint64, _VP, C.c_int, _VP]),
    ("mt_brdf_batch", C.c_int, [_VP, C.c_uint64, _VP]),
    ("mt_brdf_sample_batch", C.c_int, [_VP, C.c_uint64, _VP]),
    ("mt_resolve_batch", C.c_int, [_VP, C.c_uint32, C.c_uint32, C.c_int, C.c_float, C.c_int, _VP]),
    ("mt_bvh_build", C.c_int, [_VP, C.c_uint32, C.c_uint32, C.c_uint32, C.POINTER(C.POINTER(mt_bvh_node)),
                               C.POINTER(C.c_uint32), C.POINTER(C.POINTER(C.c_uint32)), C.POINTER(C.c_uint32)]),
    ("mt_bvh_free", None, [_VP, _VP]),
    ("mt_image_rgb8", C.c_int, [_VP, C.c_uint32, C.c_uint32, _VP, _VP]),
    ("mt_write_png", C.c_int, [C.c_char_p, _VP, C.c_uint32, C.c_uint32]),
    ("mt_write_hdr", C.c_int, [C.c_char_p, _VP, C.c_uint32, C.c_uint32]),
    ("mt_last_error", C.c_char_p, []),
    ("mt_abi_version", C.c_int, []),
    ("mt_kernel_launches", C.c_uint64, [_VP]),
    ("mt_profile_enable", C.c_int, [_VP, C.c_int, C.c_int]),
    ("mt_profile_read", C.c_int, [_VP, C.POINTER(mt_profile)]),
    ("mt_profile_reset", C.c_int, [_VP]),
]


def _load():
    if not LIB_PATH.exists():
        raise ImportError(
            f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
            "(the CUDA kernels are the only implementation; there is no CPU fallback)"
        )
    lib = C.CDLL(str(LIB_PATH))
    for name, res, args in PROTOTYPES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


lib = _load()


class MTError(RuntimeError):
    def __init__(self, code: int, where: str):
        msg = lib.mt_last_error().decode(errors="replace")
        super().__init__(f"{where}: {STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


def check(code: int, where: str):
    if code != MT_OK:
        raise MTError(code, where)
