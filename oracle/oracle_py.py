"""ctypes binding of the CPU oracle (oracle/oracle.h).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's cpu_baseline / --impl reference legs.  The product never imports it.
Parity against the reference's own outputs is unpinned (the reference cannot be
built here and ships no golden vectors); the oracle is pinned by the
known-answer tests under tests/.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
RNG_MT19937, RNG_COUNTER = 0, 1


def _build_if_needed():
    import subprocess

    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)


def load(fast: bool = False):
    name = "liboracle_fast.so" if fast else "liboracle.so"
    path = HERE / name
    if not path.exists():
        _build_if_needed()
    lib = C.CDLL(str(path))
    vp = C.c_void_p
    protos = {
        "orc_bvh_build": (C.c_int, [vp, C.c_uint32, C.c_uint32, C.c_uint32, C.POINTER(vp), C.POINTER(C.c_uint32),
                                    C.POINTER(vp), C.POINTER(C.c_uint32)]),
        "orc_free": (None, [vp]),
        "orc_scene_create": (C.c_int, [vp, vp, C.POINTER(vp)]),
        "orc_scene_destroy": (None, [vp]),
        "orc_scene_mesh_bvh": (C.c_int, [vp, C.c_uint32, C.POINTER(vp), C.POINTER(C.c_uint32), C.POINTER(vp),
                                         C.POINTER(C.c_uint32)]),
        "orc_trace_rays": (C.c_int, [vp, vp, C.c_uint64, vp, C.c_int, vp, C.c_int]),
        "orc_trace_f64": (C.c_int, [vp, vp, vp, C.c_uint64, vp]),
        "orc_brdf_batch": (C.c_int, [vp, C.c_uint64, vp]),
        "orc_brdf_sample": (C.c_int, [vp, C.c_uint64, vp]),
        "orc_camera_rays": (C.c_int, [vp, vp, C.c_uint64, vp]),
        "orc_philox": (None, [vp, vp, vp]),
        "orc_render": (C.c_int, [vp, C.c_int, C.c_int, C.c_uint32, C.c_uint32, vp, C.POINTER(C.c_uint64),
                                 C.POINTER(C.c_uint64)]),
        "orc_render_samples": (C.c_int, [vp, C.c_int, C.c_uint32, C.c_uint32, vp]),
        "orc_resolve_pixel": (C.c_int, [vp, C.c_uint32, C.c_int, C.c_float, C.c_int, vp]),
        "orc_aces": (None, [vp, C.c_float, vp]),
        "orc_render_grad": (C.c_int, [vp, vp, vp, vp, vp, vp, vp, vp, vp, C.c_int]),
        "orc_last_error": (C.c_char_p, []),
    }
    for k, (r, a) in protos.items():
        f = getattr(lib, k)
        f.restype = r
        f.argtypes = a
    return lib


_LIBS = {}


def lib(fast: bool = False):
    if fast not in _LIBS:
        _LIBS[fast] = load(fast)
    return _LIBS[fast]


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def _check(rc, L, where):
    if rc != 0:
        raise RuntimeError(f"{where}: {rc}: {L.orc_last_error().decode()}")


def bvh_build(positions: np.ndarray, max_triangles=32, max_depth=32):
    L = lib()
    pos = np.ascontiguousarray(positions, dtype=np.float32)
    nodes, idx = C.c_void_p(), C.c_void_p()
    nn, ni = C.c_uint32(), C.c_uint32()
    _check(L.orc_bvh_build(_p(pos), pos.shape[0], max_triangles, max_depth, C.byref(nodes), C.byref(nn),
                           C.byref(idx), C.byref(ni)), L, "orc_bvh_build")
    try:
        n = np.ctypeslib.as_array(C.cast(nodes, C.POINTER(C.c_uint32)), shape=(nn.value * 8,)).reshape(-1, 8).copy()
        i = np.ctypeslib.as_array(C.cast(idx, C.POINTER(C.c_uint32)), shape=(max(ni.value, 1),))[: ni.value].copy()
    finally:
        L.orc_free(nodes)
        L.orc_free(idx)
    return n, i


def philox(ctr, key):
    L = lib()
    c = np.asarray(ctr, dtype=np.uint32)
    k = np.asarray(key, dtype=np.uint32)
    o = np.zeros(4, dtype=np.uint32)
    L.orc_philox(_p(c), _p(k), _p(o))
    return o


def brdf_batch(q: np.ndarray) -> np.ndarray:
    L = lib()
    q = np.ascontiguousarray(q, dtype=np.float32)
    out = np.zeros((q.shape[0], 5), dtype=np.float32)
    _check(L.orc_brdf_batch(_p(q), q.shape[0], _p(out)), L, "orc_brdf_batch")
    return out


def brdf_sample(q: np.ndarray) -> np.ndarray:
    """q: (n, 16) float32 in mt_brdf_sample_query layout -> (n, 6) float32 rows
    (L xyz, pdf, specular probability, lobe as int32 bits)."""
    L = lib()
    q = np.ascontiguousarray(q, dtype=np.float32)
    out = np.zeros((q.shape[0], 6), dtype=np.float32)
    _check(L.orc_brdf_sample(_p(q), q.shape[0], _p(out)), L, "orc_brdf_sample")
    return out


def aces(rgb, exposure):
    L = lib()
    a = np.asarray(rgb, dtype=np.float32)
    o = np.zeros(3, dtype=np.float32)
    L.orc_aces(_p(a), float(exposure), _p(o))
    return o


def resolve_pixel(samples: np.ndarray, enable=True, k=6.0, debug_mode=0):
    L = lib()
    s = np.ascontiguousarray(samples, dtype=np.float32)
    o = np.zeros(3, dtype=np.float32)
    _check(L.orc_resolve_pixel(_p(s), s.shape[0], int(enable), float(k), int(debug_mode), _p(o)), L,
           "orc_resolve_pixel")
    return o


class OracleScene:
    """The oracle's copy of a scene; takes the same PackedScene / mt_config the
    product takes (the boundary format)."""

    def __init__(self, packed, cfg, fast: bool = False):
        self.L = lib(fast)
        self.packed = packed
        self.cfg = cfg
        h = C.c_void_p()
        _check(self.L.orc_scene_create(C.cast(packed.ptr(), C.c_void_p), C.cast(C.byref(cfg), C.c_void_p),
                                       C.byref(h)), self.L, "orc_scene_create")
        self.h = h

    def close(self):
        if self.h:
            self.L.orc_scene_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def mesh_bvh(self, mesh: int):
        nodes, idx = C.c_void_p(), C.c_void_p()
        nn, ni = C.c_uint32(), C.c_uint32()
        _check(self.L.orc_scene_mesh_bvh(self.h, mesh, C.byref(nodes), C.byref(nn), C.byref(idx), C.byref(ni)),
               self.L, "orc_scene_mesh_bvh")
        if nn.value == 0:
            return None, None
        n = np.ctypeslib.as_array(C.cast(nodes, C.POINTER(C.c_uint32)), shape=(nn.value * 8,)).reshape(-1, 8).copy()
        i = np.ctypeslib.as_array(C.cast(idx, C.POINTER(C.c_uint32)), shape=(ni.value,)).copy()
        return n, i

    def trace(self, rays: np.ndarray, query=0, totals=False, threads=0):
        rays = np.ascontiguousarray(rays, dtype=np.float32)
        hits = np.zeros((rays.shape[0], 8), dtype=np.uint32)
        tot = np.zeros((rays.shape[0], 3), dtype=np.uint32) if totals else None
        _check(self.L.orc_trace_rays(self.h, _p(rays), rays.shape[0], _p(hits), query,
                                     _p(tot) if totals else None, threads), self.L, "orc_trace_rays")
        return (hits, tot) if totals else hits

    def trace_f64(self, rays: np.ndarray, hits: np.ndarray) -> np.ndarray:
        rays = np.ascontiguousarray(rays, dtype=np.float32)
        hits = np.ascontiguousarray(hits, dtype=np.uint32)
        out = np.zeros((rays.shape[0], 3), dtype=np.float64)
        _check(self.L.orc_trace_f64(self.h, _p(rays), _p(hits), rays.shape[0], _p(out)), self.L, "orc_trace_f64")
        return out

    def camera_rays(self, uv: np.ndarray) -> np.ndarray:
        uv = np.ascontiguousarray(uv, dtype=np.float32)
        out = np.zeros((uv.shape[0], 8), dtype=np.float32)
        _check(self.L.orc_camera_rays(self.h, _p(uv), uv.shape[0], _p(out)), self.L, "orc_camera_rays")
        return out

    def render(self, rng=RNG_COUNTER, threads=0, row0=0, row1=None):
        W, H = self.cfg.width, self.cfg.height
        row1 = H if row1 is None else row1
        img = np.zeros((H, W, 3), dtype=np.float32)
        rays, samples = C.c_uint64(), C.c_uint64()
        _check(self.L.orc_render(self.h, rng, threads, row0, row1, _p(img), C.byref(rays), C.byref(samples)),
               self.L, "orc_render")
        return img, rays.value, samples.value

    def render_grad(self, target: np.ndarray, num_texels: int = 0, threads=0):
        """Counter-RNG render plus dL/dparameters of L = sum (image - target)^2.
        Returns dict(image, loss, d_base (M,3), d_roughness (M,), d_metallic (M,),
        d_light (Lights,), d_texels (num_texels,))."""
        cfg = self.cfg
        target = np.ascontiguousarray(target, dtype=np.float32).reshape(cfg.height, cfg.width, 3)
        nm = self.packed.desc.num_materials
        nl = self.packed.desc.num_lights
        out = {
            "image": np.zeros((cfg.height, cfg.width, 3), np.float32),
            "loss": np.zeros(1, np.float32),
            "d_base": np.zeros((nm, 3), np.float32),
            "d_roughness": np.zeros(nm, np.float32),
            "d_metallic": np.zeros(nm, np.float32),
            "d_light": np.zeros(max(nl, 1), np.float32),
            "d_texels": np.zeros(max(num_texels, 1), np.float32),
        }
        _check(self.L.orc_render_grad(self.h, _p(target), _p(out["image"]), _p(out["loss"]), _p(out["d_base"]),
                                      _p(out["d_roughness"]), _p(out["d_metallic"]), _p(out["d_light"]),
                                      _p(out["d_texels"]), threads), self.L, "orc_render_grad")
        out["loss"] = float(out["loss"][0])
        out["d_light"] = out["d_light"][:nl]
        out["d_texels"] = out["d_texels"][:num_texels]
        return out

    def render_samples(self, row0=0, row1=None, threads=0):
        W, H, S = self.cfg.width, self.cfg.height, self.cfg.samples
        row1 = H if row1 is None else row1
        out = np.zeros((S, row1 - row0, W, 3), dtype=np.float32)
        _check(self.L.orc_render_samples(self.h, threads, row0, row1, _p(out)), self.L, "orc_render_samples")
        return out
