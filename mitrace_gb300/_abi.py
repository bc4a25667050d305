"""ctypes mirror of ``include/mitrace_gpu.h`` and the loader of the in-tree
``libmitrace_gb300.so``.

There is no fallback: if the shared library is missing or fails to load, the
import of this module raises, so nothing can silently run without the CUDA
kernels.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libmitrace_gb300.so"

MT_OK, MT_ERR_CUDA, MT_ERR_OOM, MT_ERR_INVALID, MT_ERR_TIMEOUT, MT_ERR_KILLED, MT_ERR_STATE = range(7)
STATUS_NAMES = {
    0: "MT_OK",
    1: "MT_ERR_CUDA",
    2: "MT_ERR_OOM",
    3: "MT_ERR_INVALID",
    4: "MT_ERR_TIMEOUT",
    5: "MT_ERR_KILLED",
    6: "MT_ERR_STATE",
}
MT_BVH_LEAF_BIT = 0x80000000
MT_NO_HIT = 0xFFFFFFFF
MT_QUERY_CLOSEST, MT_QUERY_ANY, MT_QUERY_CLOSEST_COUNT = 0, 1, 2
MT_FILTER_NEAREST, MT_FILTER_LINEAR = 0, 1
MT_LIGHT_POINT, MT_LIGHT_DIRECTIONAL, MT_LIGHT_SPOT, MT_LIGHT_AREA = 0, 1, 2, 3


class mt_bvh_node(C.Structure):
    _fields_ = [("lo", C.c_float * 3), ("hi", C.c_float * 3), ("a", C.c_uint32), ("b", C.c_uint32)]


class mt_mesh_desc(C.Structure):
    _fields_ = [
        ("num_triangles", C.c_uint32),
        ("positions", C.POINTER(C.c_float)),
        ("normals", C.POINTER(C.c_float)),
        ("uv0", C.POINTER(C.c_float)),
        ("bvh_nodes", C.POINTER(mt_bvh_node)),
        ("num_bvh_nodes", C.c_uint32),
        ("bvh_indices", C.POINTER(C.c_uint32)),
        ("num_bvh_indices", C.c_uint32),
    ]


class mt_texture_desc(C.Structure):
    _fields_ = [
        ("width", C.c_uint32),
        ("height", C.c_uint32),
        ("rgb8", C.POINTER(C.c_uint8)),
        ("rgb32f", C.POINTER(C.c_float)),
        ("filter", C.c_int32),
        ("offset", C.c_float * 2),
        ("scale", C.c_float * 2),
    ]


class mt_material_desc(C.Structure):
    _fields_ = [
        ("base_color_factor", C.c_float * 4),
        ("emissive_factor", C.c_float * 3),
        ("normal_scale", C.c_float),
        ("metallic_factor", C.c_float),
        ("roughness_factor", C.c_float),
        ("occlusion_strength", C.c_float),
        ("base_color_tex", C.c_int32),
        ("metallic_roughness_tex", C.c_int32),
        ("normal_tex", C.c_int32),
        ("occlusion_tex", C.c_int32),
        ("emissive_tex", C.c_int32),
    ]


class mt_instance_desc(C.Structure):
    _fields_ = [("mesh", C.c_uint32), ("material", C.c_uint32), ("transform", C.c_float * 16)]


class mt_light_desc(C.Structure):
    _fields_ = [
        ("type", C.c_int32),
        ("position", C.c_float * 3),
        ("color", C.c_float * 3),
        ("point_size", C.c_float),
        ("spot_inner_cos", C.c_float),
        ("spot_outer_cos", C.c_float),
        ("direction", C.c_float * 3),
    ]


class mt_camera_desc(C.Structure):
    _fields_ = [
        ("type", C.c_int32),
        ("camera_to_world", C.c_float * 16),
        ("yfov", C.c_float),
        ("aspect", C.c_float),
        ("ortho_size", C.c_float * 2),
    ]


class mt_scene_desc(C.Structure):
    _fields_ = [
        ("num_meshes", C.c_uint32),
        ("meshes", C.POINTER(mt_mesh_desc)),
        ("num_instances", C.c_uint32),
        ("instances", C.POINTER(mt_instance_desc)),
        ("num_materials", C.c_uint32),
        ("materials", C.POINTER(mt_material_desc)),
        ("num_textures", C.c_uint32),
        ("textures", C.POINTER(mt_texture_desc)),
        ("num_lights", C.c_uint32),
        ("lights", C.POINTER(mt_light_desc)),
        ("camera", mt_camera_desc),
        ("env_texture", C.c_int32),
    ]


class mt_config(C.Structure):
    _fields_ = [
        ("width", C.c_uint32),
        ("height", C.c_uint32),
        ("samples", C.c_uint32),
        ("bounces", C.c_uint32),
        ("ev_exposure", C.c_float),
        ("hdri_primary_intensity", C.c_float),
        ("hdri_secondary_intensity", C.c_float),
        ("emission_base_intensity", C.c_float),
        ("bvh_disable", C.c_int32),
        ("bvh_max_triangles", C.c_uint32),
        ("bvh_max_depth", C.c_uint32),
        ("firefly_enable", C.c_int32),
        ("firefly_threshold", C.c_float),
        ("terminate_energy", C.c_float),
        ("debug_mode", C.c_int32),
        ("reserved0", C.c_uint32),
        ("seed", C.c_uint64),
        ("reserved", C.c_uint32 * 8),
    ]


class mt_stats(C.Structure):
    _fields_ = [
        ("progress", C.c_float),
        ("time_elapsed", C.c_float),
        ("estimated_time_remaining", C.c_float),
        ("reserved", C.c_float),
        ("rays", C.c_uint64),
        ("samples", C.c_uint64),
    ]


class mt_ray(C.Structure):
    _fields_ = [("origin", C.c_float * 3), ("tmax", C.c_float), ("direction", C.c_float * 3), ("pad", C.c_float)]


class mt_hit(C.Structure):
    _fields_ = [
        ("distance", C.c_float),
        ("u", C.c_float),
        ("v", C.c_float),
        ("instance", C.c_uint32),
        ("triangle", C.c_uint32),
        ("bv_index", C.c_uint32),
        ("bvh_tests", C.c_uint32),
        ("tri_tests", C.c_uint32),
    ]


class mt_stage_profile(C.Structure):
    _fields_ = [
        ("launches", C.c_uint64),
        ("milliseconds", C.c_double),
        ("rays", C.c_uint64),
        ("node_pops", C.c_uint64),
        ("inner_pops", C.c_uint64),
        ("tri_tests", C.c_uint64),
    ]


MT_STAGE_RAYGEN, MT_STAGE_EXTEND, MT_STAGE_SHADE, MT_STAGE_SHADOW, MT_STAGE_FINALIZE, MT_STAGE_RESOLVE = range(6)
MT_NUM_STAGES = 6
MT_QUERY_CLOSEST_TOTALS = 3
MT_NOALLOC_MAX_PATHS = 65536
MT_NOALLOC_SCRATCH_BYTES = 16 << 20


class mt_profile(C.Structure):
    _fields_ = [("stage", mt_stage_profile * MT_NUM_STAGES)]


class mt_grad_buffers(C.Structure):
    _fields_ = [
        ("target", C.c_void_p),
        ("image", C.c_void_p),
        ("loss", C.c_void_p),
        ("d_base", C.c_void_p),
        ("d_roughness", C.c_void_p),
        ("d_metallic", C.c_void_p),
        ("d_light", C.c_void_p),
        ("d_texels", C.c_void_p),
        ("d_image", C.c_void_p),
    ]


MT_GRAD_MAX_BOUNCES = 16

MT_NRC_INPUTS = 80
MT_NRC_WIDTH = 64
MT_NRC_FEATURES = 20
MT_NRC_PARAMS = 80 * 64 + 3 * 64 * 64 + 64 * 3
MT_NRC_END_AFTER_DIFFUSE = 0
MT_NRC_END_AT_DIFFUSE = 1


class mt_nrc_config(C.Structure):
    _fields_ = [
        ("train_paths", C.c_uint32),
        ("train_batch", C.c_uint32),
        ("train_steps", C.c_uint32),
        ("spp", C.c_uint32),
        ("learning_rate", C.c_float),
        ("beta1", C.c_float),
        ("beta2", C.c_float),
        ("epsilon", C.c_float),
        ("rough_min", C.c_float),
        ("seed", C.c_uint32),
        ("ema_decay", C.c_float),
        ("end_at", C.c_uint32),
        ("target_cap", C.c_float),
        ("reserved", C.c_uint32 * 3),
    ]


class mt_nrc_stats(C.Structure):
    _fields_ = [
        ("frames", C.c_uint64),
        ("adam_steps", C.c_uint64),
        ("train_samples", C.c_uint32),
        ("queries", C.c_uint32),
        ("train_loss", C.c_float),
        ("reserved", C.c_float * 3),
    ]


class mt_brdf_query(C.Structure):
    _fields_ = [
        ("L", C.c_float * 3),
        ("V", C.c_float * 3),
        ("N", C.c_float * 3),
        ("base_color", C.c_float * 3),
        ("roughness", C.c_float),
        ("metallic", C.c_float),
    ]


class mt_brdf_result(C.Structure):
    _fields_ = [("f", C.c_float * 3), ("diffuse_pdf", C.c_float), ("specular_pdf", C.c_float)]


class mt_brdf_sample_query(C.Structure):
    _fields_ = [("V", C.c_float * 3), ("N", C.c_float * 3), ("base_color", C.c_float * 3), ("roughness", C.c_float),
                ("metallic", C.c_float), ("u", C.c_float * 5)]


class mt_brdf_sample_result(C.Structure):
    _fields_ = [("L", C.c_float * 3), ("pdf", C.c_float), ("specular_probability", C.c_float),
                ("lobe", C.c_int32)]


# Every entry point declared in include/mitrace_gpu.h: (name, restype, argtypes).
_VP = C.c_void_p
PROTOTYPES = [
    ("mt_config_defaults", None, [C.POINTER(mt_config)]),
    ("mt_create", C.c_int, [C.POINTER(mt_scene_desc), C.POINTER(mt_config), C.POINTER(_VP)]),
    ("mt_destroy", None, [_VP]),
    ("mt_start", C.c_int, [_VP]),
    ("mt_wait", C.c_int, [_VP, _VP]),
    ("mt_kill", C.c_int, [_VP]),
    ("mt_get_stats", C.c_int, [_VP, C.POINTER(mt_stats)]),
    ("mt_is_done", C.c_int, [_VP]),
    ("mt_render_device", C.c_int, [_VP, _VP, _VP]),
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
