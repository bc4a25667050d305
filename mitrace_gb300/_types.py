"""ctypes mirror of the types and constants of ``include/mitrace_gpu.h``.

Pure Python: importing this module loads no library, so the synthetic scene
generators (``scenes.py``) can build boundary structs in a process that never
maps ``libmitrace_gb300.so`` (the CPU reference arm of the benchmark).
``_abi.py`` re-exports everything here and loads the library.
"""
from __future__ import annotations

import ctypes as C

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


MT_DEBUG_PIXEL_STANDARD_DEVIATION = 21
MT_DEBUG_FIREFLY_ELIMINATION = 22
MT_DEBUG_COUNT = 23


def config_defaults(c: mt_config) -> mt_config:
    """Fills c with the reference's Config defaults (src/CLI/Config.hpp:48-70),
    the values mt_config_defaults writes (a CPU test keeps the two equal)."""
    C.memset(C.byref(c), 0, C.sizeof(c))
    c.width, c.height, c.samples, c.bounces = 1280, 720, 64, 5
    c.ev_exposure = 8.0
    c.hdri_primary_intensity = 350.0
    c.hdri_secondary_intensity = 350.0
    c.emission_base_intensity = 1.0
    c.bvh_disable = 0
    c.bvh_max_triangles = 32
    c.bvh_max_depth = 32
    c.firefly_enable = 1
    c.firefly_threshold = 6.0
    c.terminate_energy = 0.01
    c.debug_mode = 0
    c.seed = 0
    return c
