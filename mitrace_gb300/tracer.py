"""Python view of the C ABI, shaped like MiTrace's ``Tracer::Tracer``
(src/Tracer/Tracer.hpp:121-128): construct with a scene, ``StartRender`` (non
blocking), ``WaitForRender``, ``KillRender``, ``GetStats``, ``IsDone``.  The
image lands in a ``RenderBuffer``-like float32 array (H, W, 3) of tonemapped
means (src/Tracer/RenderBuffer.hpp:11-35).

Also exposes the ray-query and BRDF test entry points.  Every call goes to
``libmitrace_gb300.so``; there is no other implementation.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _abi as A
from .scenes import PackedScene, SceneData


@dataclass
class Stats:
    progress: float
    timeElapsed: float
    estimatedTimeRemaining: float
    rays: int
    samples: int


class Tracer:
    def __init__(self, scene: SceneData, config: A.mt_config, packed: PackedScene = None):
        """mt_create over the scene's host arrays.  `packed` (a PackedScene of
        the same scene) saves re-building the C descriptor structs when one
        scene is handed to many tracers; the data is uploaded either way."""
        self.scene = scene
        self.config = config
        self._packed = packed if packed is not None else PackedScene(scene)
        h = C.c_void_p()
        A.check(A.lib.mt_create(self._packed.ptr(), C.byref(config), C.byref(h)), "mt_create")
        self.handle = h
        self.width, self.height = config.width, config.height
        self.image = np.zeros((self.height, self.width, 3), dtype=np.float32)

    # --- reference-shaped API ------------------------------------------------
    def StartRender(self):
        A.check(A.lib.mt_start(self.handle), "mt_start")

    def WaitForRender(self, out: np.ndarray = None) -> np.ndarray:
        """mt_wait; the image lands in `out` (a C-contiguous float32 H x W x 3
        host array, e.g. pinned memory) or in the tracer's own buffer."""
        dst = self.image if out is None else out
        if out is not None:
            assert out.dtype == np.float32 and out.flags.c_contiguous and out.size == self.image.size
        A.check(A.lib.mt_wait(self.handle, dst.ctypes.data_as(C.c_void_p)), "mt_wait")
        return dst

    def KillRender(self):
        A.check(A.lib.mt_kill(self.handle), "mt_kill")

    def GetStats(self) -> Stats:
        s = A.mt_stats()
        A.check(A.lib.mt_get_stats(self.handle, C.byref(s)), "mt_get_stats")
        return Stats(s.progress, s.time_elapsed, s.estimated_time_remaining, s.rays, s.samples)

    def IsDone(self) -> bool:
        return bool(A.lib.mt_is_done(self.handle))

    # --- device-resident entry points ------------------------------------------
    def render_device(self, out_ptr: int, stream_ptr: int = 0):
        A.check(A.lib.mt_render_device(self.handle, C.c_void_p(out_ptr), C.c_void_p(stream_ptr)), "mt_render_device")

    def set_seed(self, seed: int):
        A.check(A.lib.mt_set_seed(self.handle, seed), "mt_set_seed")

    def render_rows_device(self, row0: int, row1: int, out_ptr: int, stream_ptr: int = 0):
        A.check(A.lib.mt_render_rows_device(self.handle, row0, row1, C.c_void_p(out_ptr), C.c_void_p(stream_ptr)),
                "mt_render_rows_device")

    def trace_device(self, rays_ptr: int, n: int, hits_ptr: int, query: int = A.MT_QUERY_CLOSEST, stream_ptr: int = 0):
        A.check(A.lib.mt_trace_rays_device(self.handle, C.c_void_p(rays_ptr), n, C.c_void_p(hits_ptr), query,
                                           C.c_void_p(stream_ptr)), "mt_trace_rays_device")

    def trace(self, rays: np.ndarray, query: int = A.MT_QUERY_CLOSEST) -> np.ndarray:
        """rays: (n, 8) float32 in mt_ray layout.  Returns an (n, 8) uint32 view
        of mt_hit records (distance/u/v are float bits)."""
        rays = np.ascontiguousarray(rays, dtype=np.float32)
        assert rays.ndim == 2 and rays.shape[1] == 8
        hits = np.zeros((rays.shape[0], 8), dtype=np.uint32)
        A.check(A.lib.mt_trace_rays(self.handle, rays.ctypes.data_as(C.c_void_p), rays.shape[0],
                                    hits.ctypes.data_as(C.c_void_p), query), "mt_trace_rays")
        return hits

    def render_grad_device(self, target_ptr: int, image_ptr: int, loss_ptr: int, d_base_ptr: int,
                           d_rough_ptr: int, d_metal_ptr: int, d_light_ptr: int, d_texels_ptr: int = 0,
                           stream_ptr: int = 0, d_image_ptr: int = 0):
        """mt_render_grad on device buffers (gradients are added to the d_* buffers);
        with d_image_ptr the image gradient is given instead of a target."""
        g = A.mt_grad_buffers(target_ptr or None, image_ptr, loss_ptr or None, d_base_ptr, d_rough_ptr, d_metal_ptr,
                              d_light_ptr or None, d_texels_ptr or None, d_image_ptr or None)
        A.check(A.lib.mt_render_grad(self.handle, C.byref(g), C.c_void_p(stream_ptr)), "mt_render_grad")

    # --- parameter updates (inverse rendering) -----------------------------------
    def update_materials(self, materials):
        """mt_update_materials: new factors for every material (same texture slots)."""
        ps = PackedScene(SceneData(meshes=[], instances=[], materials=list(materials)))
        A.check(A.lib.mt_update_materials(self.handle, C.cast(ps.desc.materials, C.c_void_p), len(materials)),
                "mt_update_materials")

    def update_lights(self, lights):
        """mt_update_lights: new positions / colours for every light (same types)."""
        ps = PackedScene(SceneData(meshes=[], instances=[], materials=[], lights=list(lights)))
        A.check(A.lib.mt_update_lights(self.handle, C.cast(ps.desc.lights, C.c_void_p), len(lights)),
                "mt_update_lights")

    def update_texture(self, index: int, texels: np.ndarray):
        """mt_update_texture: all texels of one texture (same size and format)."""
        a = np.ascontiguousarray(texels)
        A.check(A.lib.mt_update_texture(self.handle, index, a.ctypes.data_as(C.c_void_p)), "mt_update_texture")

    # --- neural radiance cache ---------------------------------------------------
    def nrc_enable(self, **overrides) -> A.mt_nrc_config:
        """mt_nrc_enable with mt_nrc_config_defaults plus the given fields."""
        c = A.mt_nrc_config()
        A.lib.mt_nrc_config_defaults(C.byref(c))
        for k, v in overrides.items():
            setattr(c, k, v)
        A.check(A.lib.mt_nrc_enable(self.handle, C.byref(c)), "mt_nrc_enable")
        self.nrc_config = c
        return c

    def nrc_frame(self, accum_ptr: int = 0, accum_index: int = 0, stream_ptr: int = 0):
        """One training iteration plus (accum_ptr != 0) one cached frame folded
        into the running mean at accum_ptr (W*H*3 float32 on the device)."""
        A.check(A.lib.mt_nrc_frame(self.handle, C.c_void_p(accum_ptr or None), accum_index,
                                   C.c_void_p(stream_ptr)), "mt_nrc_frame")

    def nrc_get_stats(self) -> dict:
        st = A.mt_nrc_stats()
        A.check(A.lib.mt_nrc_get_stats(self.handle, C.byref(st)), "mt_nrc_get_stats")
        return {"frames": st.frames, "adam_steps": st.adam_steps, "train_samples": st.train_samples,
                "queries": st.queries, "train_loss": st.train_loss}

    def nrc_get_params(self) -> np.ndarray:
        p = np.zeros(A.MT_NRC_PARAMS, dtype=np.float32)
        A.check(A.lib.mt_nrc_get_params(self.handle, p.ctypes.data_as(C.c_void_p)), "mt_nrc_get_params")
        return p

    def nrc_set_params(self, params: np.ndarray):
        p = np.ascontiguousarray(params, dtype=np.float32)
        assert p.size == A.MT_NRC_PARAMS
        A.check(A.lib.mt_nrc_set_params(self.handle, p.ctypes.data_as(C.c_void_p)), "mt_nrc_set_params")

    def nrc_infer_device(self, feat_ptr: int, n: int, out_ptr: int, stream_ptr: int = 0):
        A.check(A.lib.mt_nrc_infer(self.handle, C.c_void_p(feat_ptr), n, C.c_void_p(out_ptr),
                                   C.c_void_p(stream_ptr)), "mt_nrc_infer")

    def nrc_train_step_device(self, feat_ptr: int, target_ptr: int, n: int, loss_ptr: int = 0, grad_ptr: int = 0,
                              stream_ptr: int = 0):
        A.check(A.lib.mt_nrc_train_step(self.handle, C.c_void_p(feat_ptr), C.c_void_p(target_ptr), n,
                                        C.c_void_p(loss_ptr or None), C.c_void_p(grad_ptr or None),
                                        C.c_void_p(stream_ptr)), "mt_nrc_train_step")

    def kernel_launches(self) -> int:
        return int(A.lib.mt_kernel_launches(self.handle))

    def close(self):
        if getattr(self, "handle", None):
            A.lib.mt_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def brdf_batch(q: np.ndarray) -> np.ndarray:
    """q: (n, 14) float32 in mt_brdf_query layout -> (n, 5) float32 results."""
    q = np.ascontiguousarray(q, dtype=np.float32)
    assert q.ndim == 2 and q.shape[1] == 14
    out = np.zeros((q.shape[0], 5), dtype=np.float32)
    A.check(A.lib.mt_brdf_batch(q.ctypes.data_as(C.c_void_p), q.shape[0], out.ctypes.data_as(C.c_void_p)),
            "mt_brdf_batch")
    return out


def brdf_sample_batch(q: np.ndarray) -> np.ndarray:
    """q: (n, 16) float32 in mt_brdf_sample_query layout -> (n, 6) float32 rows
    (L xyz, pdf, specular probability, lobe as int32 bits)."""
    q = np.ascontiguousarray(q, dtype=np.float32)
    assert q.ndim == 2 and q.shape[1] == 16
    out = np.zeros((q.shape[0], 6), dtype=np.float32)
    A.check(A.lib.mt_brdf_sample_batch(q.ctypes.data_as(C.c_void_p), q.shape[0], out.ctypes.data_as(C.c_void_p)),
            "mt_brdf_sample_batch")
    return out


def image_rgb8_device(rgb_ptr: int, width: int, height: int, out_ptr: int, stream_ptr: int = 0):
    """FloatToU8 of a device image (W*H*3 floats -> bytes) on the GPU."""
    A.check(A.lib.mt_image_rgb8(C.c_void_p(rgb_ptr), width, height, C.c_void_p(out_ptr), C.c_void_p(stream_ptr)),
            "mt_image_rgb8")


def write_png(path, rgb8: np.ndarray):
    """Writes an (H, W, 3) uint8 image as PNG."""
    a = np.ascontiguousarray(rgb8, dtype=np.uint8)
    A.check(A.lib.mt_write_png(str(path).encode(), a.ctypes.data_as(C.c_void_p), a.shape[1], a.shape[0]),
            "mt_write_png")


def write_hdr(path, rgb: np.ndarray):
    """Writes an (H, W, 3) float32 image as Radiance HDR."""
    a = np.ascontiguousarray(rgb, dtype=np.float32)
    A.check(A.lib.mt_write_hdr(str(path).encode(), a.ctypes.data_as(C.c_void_p), a.shape[1], a.shape[0]),
            "mt_write_hdr")


def nrc_encode_device(feat_ptr: int, n: int, out_ptr: int, stream_ptr: int = 0):
    """The radiance cache's FP32 input encoding: n x 20 features -> n x 80 (device buffers)."""
    A.check(A.lib.mt_nrc_encode(C.c_void_p(feat_ptr), n, C.c_void_p(out_ptr), C.c_void_p(stream_ptr)),
            "mt_nrc_encode")


def bvh_build(positions: np.ndarray, max_triangles=32, max_depth=32):
    """Host BVH build of one mesh (T, 3, 3) -> ((N, 8) uint32 nodes, (M,) uint32 indices)."""
    pos = np.ascontiguousarray(positions, dtype=np.float32)
    nodes = C.POINTER(A.mt_bvh_node)()
    idx = C.POINTER(C.c_uint32)()
    nn, ni = C.c_uint32(), C.c_uint32()
    A.check(A.lib.mt_bvh_build(pos.ctypes.data_as(C.c_void_p), pos.shape[0], max_triangles, max_depth,
                               C.byref(nodes), C.byref(nn), C.byref(idx), C.byref(ni)), "mt_bvh_build")
    try:
        n = np.ctypeslib.as_array(C.cast(nodes, C.POINTER(C.c_uint32)), shape=(nn.value * 8,)).reshape(-1, 8).copy()
        i = np.ctypeslib.as_array(idx, shape=(max(ni.value, 1),))[: ni.value].copy()
    finally:
        A.lib.mt_bvh_free(C.cast(nodes, C.c_void_p), C.cast(idx, C.c_void_p))
    return n, i
