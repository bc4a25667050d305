"""Scene data in the boundary format (``mt_scene_desc``) and the seeded synthetic
scenes the renderer is measured on.

The reference loads glTF into ``Scene::Scene`` (src/Scene/Scene.cpp:53-59); the
drop-in boundary takes the flattened result of that step.  The generators
below build the same kind of data directly in memory (no dataset, no network):

* ``box_room``       - 34-triangle box room with one point light, 256x256.
* ``material_grid``  - 7x7 UV spheres (4096 triangles each) on a ground plane,
                       procedural float sky with a sun disk, 2 point lights, 1080p.
* ``large_scene``    - fBm terrain plus scattered icospheres (merged meshes) with
                       procedural 2048^2 base-colour / normal maps.
* ``incoherent_rays``- origins uniform in a box, directions uniform on the sphere.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field
from typing import List, Optional, Tuple

import numpy as np

from . import _types as A

# ----------------------------------------------------------------------------
# Data classes
# ----------------------------------------------------------------------------


@dataclass
class MeshData:
    positions: np.ndarray  # (T, 3, 3) float32, de-indexed triangles
    normals: np.ndarray  # (T, 3, 3) float32
    uv0: Optional[np.ndarray] = None  # (T, 3, 2) float32
    bvh_nodes: Optional[np.ndarray] = None  # (N, 8) uint32 view of mt_bvh_node
    bvh_indices: Optional[np.ndarray] = None  # (M,) uint32

    @property
    def num_triangles(self) -> int:
        return int(self.positions.shape[0])


@dataclass
class TextureData:
    rgb8: Optional[np.ndarray] = None  # (H, W, 3) uint8
    rgb32f: Optional[np.ndarray] = None  # (H, W, 3) float32
    filter: int = A.MT_FILTER_NEAREST
    offset: Tuple[float, float] = (0.0, 0.0)
    scale: Tuple[float, float] = (1.0, 1.0)

    @property
    def shape(self):
        t = self.rgb8 if self.rgb8 is not None else self.rgb32f
        return t.shape


@dataclass
class MaterialData:
    base_color: Tuple[float, float, float, float] = (1.0, 1.0, 1.0, 1.0)
    emissive: Tuple[float, float, float] = (0.0, 0.0, 0.0)
    normal_scale: float = 1.0
    metallic: float = 1.0
    roughness: float = 1.0
    occlusion_strength: float = 1.0
    base_tex: int = -1
    mr_tex: int = -1
    normal_tex: int = -1
    occlusion_tex: int = -1
    emissive_tex: int = -1


@dataclass
class InstanceData:
    mesh: int
    material: int
    transform: np.ndarray = field(default_factory=lambda: np.eye(4, dtype=np.float32))  # math (row-major) 4x4


@dataclass
class LightData:
    type: int = A.MT_LIGHT_POINT
    position: Tuple[float, float, float] = (0.0, 0.0, 0.0)
    color: Tuple[float, float, float] = (1.0, 1.0, 1.0)  # already multiplied by intensity
    point_size: float = 0.1
    inner_cos: float = 1.0
    outer_cos: float = 0.70710677
    direction: Tuple[float, float, float] = (0.0, 0.0, -1.0)


@dataclass
class CameraData:
    type: int = 0
    cam_to_world: np.ndarray = field(default_factory=lambda: np.eye(4, dtype=np.float32))
    yfov: float = math.radians(60.0)
    aspect: float = 1.0
    ortho: Tuple[float, float] = (0.0, 0.0)


@dataclass
class SceneData:
    meshes: List[MeshData]
    instances: List[InstanceData]
    materials: List[MaterialData]
    textures: List[TextureData] = field(default_factory=list)
    lights: List[LightData] = field(default_factory=list)
    camera: CameraData = field(default_factory=CameraData)
    env: int = -1

    @property
    def num_triangles(self) -> int:
        return sum(self.meshes[i.mesh].num_triangles for i in self.instances)

    def nbytes(self) -> int:
        n = 0
        for m in self.meshes:
            n += m.positions.nbytes + m.normals.nbytes + (m.uv0.nbytes if m.uv0 is not None else 0)
        for t in self.textures:
            n += (t.rgb8 if t.rgb8 is not None else t.rgb32f).nbytes
        return n


# ----------------------------------------------------------------------------
# Config
# ----------------------------------------------------------------------------


def make_config(**kw) -> A.mt_config:
    """mt_config with the reference defaults (Config.hpp:50-70), then overrides."""
    c = A.config_defaults(A.mt_config())
    for k, v in kw.items():
        if not hasattr(c, k):
            raise KeyError(f"unknown config field {k}")
        setattr(c, k, v)
    return c


def config_dict(c: A.mt_config) -> dict:
    return {name: getattr(c, name) for name, _ in c._fields_ if not name.startswith("reserved")}


# ----------------------------------------------------------------------------
# Packing into the C boundary structs
# ----------------------------------------------------------------------------


def _fptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _colmajor(m: np.ndarray):
    return (C.c_float * 16)(*np.asarray(m, dtype=np.float32).T.reshape(-1).tolist())


class PackedScene:
    """An ``mt_scene_desc`` whose pointers stay valid while this object lives."""

    def __init__(self, s: SceneData):
        self.keep = []
        meshes = (A.mt_mesh_desc * max(1, len(s.meshes)))()
        for i, m in enumerate(s.meshes):
            pos = np.ascontiguousarray(m.positions, dtype=np.float32)
            nrm = np.ascontiguousarray(m.normals, dtype=np.float32)
            assert pos.shape == (m.num_triangles, 3, 3) and nrm.shape == pos.shape
            self.keep += [pos, nrm]
            d = meshes[i]
            d.num_triangles = m.num_triangles
            d.positions = _fptr(pos)
            d.normals = _fptr(nrm)
            if m.uv0 is not None:
                uv = np.ascontiguousarray(m.uv0, dtype=np.float32)
                self.keep.append(uv)
                d.uv0 = _fptr(uv)
            if m.bvh_nodes is not None:
                bn = np.ascontiguousarray(m.bvh_nodes, dtype=np.uint32)
                bi = np.ascontiguousarray(m.bvh_indices, dtype=np.uint32)
                self.keep += [bn, bi]
                d.bvh_nodes = bn.ctypes.data_as(C.POINTER(A.mt_bvh_node))
                d.num_bvh_nodes = bn.shape[0]
                d.bvh_indices = bi.ctypes.data_as(C.POINTER(C.c_uint32))
                d.num_bvh_indices = bi.shape[0]
        insts = (A.mt_instance_desc * max(1, len(s.instances)))()
        for i, it in enumerate(s.instances):
            insts[i].mesh = it.mesh
            insts[i].material = it.material
            insts[i].transform = _colmajor(it.transform)
        mats = (A.mt_material_desc * max(1, len(s.materials)))()
        for i, m in enumerate(s.materials):
            d = mats[i]
            d.base_color_factor = (C.c_float * 4)(*m.base_color)
            d.emissive_factor = (C.c_float * 3)(*m.emissive)
            d.normal_scale = m.normal_scale
            d.metallic_factor = m.metallic
            d.roughness_factor = m.roughness
            d.occlusion_strength = m.occlusion_strength
            d.base_color_tex = m.base_tex
            d.metallic_roughness_tex = m.mr_tex
            d.normal_tex = m.normal_tex
            d.occlusion_tex = m.occlusion_tex
            d.emissive_tex = m.emissive_tex
        texs = (A.mt_texture_desc * max(1, len(s.textures)))()
        for i, t in enumerate(s.textures):
            d = texs[i]
            h, w, _ = t.shape
            d.width, d.height = w, h
            if t.rgb8 is not None:
                a = np.ascontiguousarray(t.rgb8, dtype=np.uint8)
                d.rgb8 = a.ctypes.data_as(C.POINTER(C.c_uint8))
            else:
                a = np.ascontiguousarray(t.rgb32f, dtype=np.float32)
                d.rgb32f = _fptr(a)
            self.keep.append(a)
            d.filter = t.filter
            d.offset = (C.c_float * 2)(*t.offset)
            d.scale = (C.c_float * 2)(*t.scale)
        lights = (A.mt_light_desc * max(1, len(s.lights)))()
        for i, l in enumerate(s.lights):
            d = lights[i]
            d.type = l.type
            d.position = (C.c_float * 3)(*l.position)
            d.color = (C.c_float * 3)(*l.color)
            d.point_size = l.point_size
            d.spot_inner_cos = l.inner_cos
            d.spot_outer_cos = l.outer_cos
            d.direction = (C.c_float * 3)(*l.direction)
        desc = A.mt_scene_desc()
        desc.num_meshes, desc.meshes = len(s.meshes), meshes
        desc.num_instances, desc.instances = len(s.instances), insts
        desc.num_materials, desc.materials = len(s.materials), mats
        desc.num_textures, desc.textures = len(s.textures), texs
        desc.num_lights, desc.lights = len(s.lights), lights
        cam = s.camera
        desc.camera.type = cam.type
        desc.camera.camera_to_world = _colmajor(cam.cam_to_world)
        desc.camera.yfov = cam.yfov
        desc.camera.aspect = cam.aspect
        desc.camera.ortho_size = (C.c_float * 2)(*cam.ortho)
        desc.env_texture = s.env
        self.keep += [meshes, insts, mats, texs, lights]
        self.desc = desc

    def ptr(self):
        return C.byref(self.desc)


# ----------------------------------------------------------------------------
# Geometry helpers
# ----------------------------------------------------------------------------


def translate(x, y, z) -> np.ndarray:
    m = np.eye(4, dtype=np.float32)
    m[:3, 3] = (x, y, z)
    return m


def quad(p0, p1, p2, p3, n):
    """Two triangles (p0,p1,p2), (p0,p2,p3) with a flat normal."""
    pos = np.array([[p0, p1, p2], [p0, p2, p3]], dtype=np.float32)
    nrm = np.broadcast_to(np.asarray(n, dtype=np.float32), (2, 3, 3)).copy()
    return pos, nrm


def box(lo, hi):
    """Axis-aligned box, 12 triangles with outward normals."""
    x0, y0, z0 = lo
    x1, y1, z1 = hi
    faces = [
        quad((x0, y0, z1), (x1, y0, z1), (x1, y1, z1), (x0, y1, z1), (0, 0, 1)),
        quad((x1, y0, z0), (x0, y0, z0), (x0, y1, z0), (x1, y1, z0), (0, 0, -1)),
        quad((x0, y0, z0), (x0, y0, z1), (x0, y1, z1), (x0, y1, z0), (-1, 0, 0)),
        quad((x1, y0, z1), (x1, y0, z0), (x1, y1, z0), (x1, y1, z1), (1, 0, 0)),
        quad((x0, y1, z1), (x1, y1, z1), (x1, y1, z0), (x0, y1, z0), (0, 1, 0)),
        quad((x0, y0, z0), (x1, y0, z0), (x1, y0, z1), (x0, y0, z1), (0, -1, 0)),
    ]
    return np.concatenate([f[0] for f in faces]), np.concatenate([f[1] for f in faces])


def uv_sphere(radius=1.0, segments=64, rings=32) -> MeshData:
    """UV sphere with segments x rings quads, each split in two triangles
    (2 * segments * rings triangles; the pole rows are degenerate)."""
    i = np.arange(segments + 1, dtype=np.float64)
    j = np.arange(rings + 1, dtype=np.float64)
    phi = 2.0 * np.pi * i / segments
    th = np.pi * j / rings
    st, ct = np.sin(th)[:, None], np.cos(th)[:, None]
    dirs = np.stack([st * np.cos(phi)[None, :], np.broadcast_to(ct, (rings + 1, segments + 1)),
                     st * np.sin(phi)[None, :]], axis=-1)  # (rings+1, seg+1, 3)
    uv = np.stack(np.meshgrid(i / segments, j / rings), axis=-1)  # (rings+1, seg+1, 2)
    a = dirs[:-1, :-1]
    b = dirs[1:, :-1]
    c = dirs[1:, 1:]
    d = dirs[:-1, 1:]
    ua, ub, uc, ud = uv[:-1, :-1], uv[1:, :-1], uv[1:, 1:], uv[:-1, 1:]
    t1 = np.stack([a, b, c], axis=2).reshape(-1, 3, 3)
    t2 = np.stack([a, c, d], axis=2).reshape(-1, 3, 3)
    u1 = np.stack([ua, ub, uc], axis=2).reshape(-1, 3, 2)
    u2 = np.stack([ua, uc, ud], axis=2).reshape(-1, 3, 2)
    n = np.concatenate([t1, t2]).astype(np.float32)
    uvs = np.concatenate([u1, u2]).astype(np.float32)
    return MeshData(positions=(n * np.float32(radius)).astype(np.float32), normals=n, uv0=uvs)


def icosphere(subdiv=1):
    """Unit icosphere: 20 * 4**subdiv triangles (80 for subdiv=1)."""
    t = (1.0 + 5 ** 0.5) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
         (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
         (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    tris = np.array([[v[a], v[b], v[c]] for a, b, c in f], dtype=np.float64)
    tris /= np.linalg.norm(tris, axis=-1, keepdims=True)
    for _ in range(subdiv):
        a, b, c = tris[:, 0], tris[:, 1], tris[:, 2]
        ab, bc, ca = a + b, b + c, c + a
        ab /= np.linalg.norm(ab, axis=-1, keepdims=True)
        bc /= np.linalg.norm(bc, axis=-1, keepdims=True)
        ca /= np.linalg.norm(ca, axis=-1, keepdims=True)
        tris = np.concatenate([np.stack([a, ab, ca], 1), np.stack([b, bc, ab], 1), np.stack([c, ca, bc], 1),
                               np.stack([ab, bc, ca], 1)])
    return tris


# ----------------------------------------------------------------------------
# Synthetic scenes
# ----------------------------------------------------------------------------


def box_room(width=256, height=256, samples=64, seed=0):
    """Box room: 2x2x2 m room of 5 quads (10 tris) + two blocks (24 tris),
    metallic 0 / roughness 1, white 0.73 / red / green walls, one 20 W point
    light of radius 0.05 under the ceiling centre, 40 degree camera.
    Render settings: terminate energy 0.1, firefly clamp 4 sigma, ev 0."""
    white = MaterialData(base_color=(0.73, 0.73, 0.73, 1.0), metallic=0.0, roughness=1.0)
    red = MaterialData(base_color=(0.65, 0.05, 0.05, 1.0), metallic=0.0, roughness=1.0)
    green = MaterialData(base_color=(0.12, 0.45, 0.15, 1.0), metallic=0.0, roughness=1.0)
    floor = quad((-1, 0, -1), (-1, 0, 1), (1, 0, 1), (1, 0, -1), (0, 1, 0))
    ceil = quad((-1, 2, -1), (1, 2, -1), (1, 2, 1), (-1, 2, 1), (0, -1, 0))
    back = quad((-1, 0, -1), (1, 0, -1), (1, 2, -1), (-1, 2, -1), (0, 0, 1))
    left = quad((-1, 0, -1), (-1, 2, -1), (-1, 2, 1), (-1, 0, 1), (1, 0, 0))
    right = quad((1, 0, -1), (1, 0, 1), (1, 2, 1), (1, 2, -1), (-1, 0, 0))
    b1 = box((0.10, 0.0, -0.25), (0.70, 0.60, 0.35))
    b2 = box((-0.72, 0.0, -0.80), (-0.12, 1.20, -0.20))
    white_walls = MeshData(np.concatenate([floor[0], ceil[0], back[0]]), np.concatenate([floor[1], ceil[1], back[1]]))
    blocks = MeshData(np.concatenate([b1[0], b2[0]]), np.concatenate([b1[1], b2[1]]))
    meshes = [white_walls, MeshData(*left), MeshData(*right), blocks]
    instances = [InstanceData(0, 0), InstanceData(1, 1), InstanceData(2, 2), InstanceData(3, 0)]
    light = LightData(type=A.MT_LIGHT_POINT, position=(0.0, 1.9, 0.0),
                      color=tuple(np.float32([1, 1, 1]) * np.float32(20.0)), point_size=0.05)
    cam = CameraData(type=0, cam_to_world=translate(0.0, 1.0, 3.4), yfov=math.radians(40.0), aspect=1.0)
    scene = SceneData(meshes, instances, [white, red, green], [], [light], cam, -1)
    cfg = make_config(width=width, height=height, samples=samples, terminate_energy=0.1, firefly_threshold=4.0,
                      ev_exposure=0.0, seed=seed)
    return scene, cfg


def sky_texture(width=512, height=256, sun_dir=(0.35, 0.8, 0.48), sun_radius_deg=2.0, sun_value=5.0e3):
    """Procedural equirectangular RGB32F sky: horizon-to-zenith gradient, dark
    ground, and a sun disk of the given value.  Rows follow
    Image::SampleEquirectangular: v = acos(y) / pi, u = (atan2(z, x) + pi) / 2pi."""
    v = (np.arange(height, dtype=np.float64) + 0.5) / height
    u = (np.arange(width, dtype=np.float64) + 0.5) / width
    phi = v * np.pi
    theta = u * 2 * np.pi - np.pi
    y = np.cos(phi)[:, None] * np.ones((1, width))
    x = np.sin(phi)[:, None] * np.cos(theta)[None, :]
    z = np.sin(phi)[:, None] * np.sin(theta)[None, :]
    up = np.clip(y, 0.0, 1.0)[..., None]
    horizon = np.array([0.85, 0.9, 1.0])
    zenith = np.array([0.25, 0.45, 0.95])
    ground = np.array([0.18, 0.16, 0.14])
    sky = np.where(y[..., None] >= 0.0, horizon * (1 - up) + zenith * up, ground)
    s = np.asarray(sun_dir, dtype=np.float64)
    s /= np.linalg.norm(s)
    cosang = x * s[0] + y * s[1] + z * s[2]
    sky[cosang > math.cos(math.radians(sun_radius_deg))] = sun_value
    return sky.astype(np.float32)


def material_grid(width=1920, height=1080, samples=256, seed=0, segments=64, rings=32):
    """7x7 UV spheres (4096 triangles each) on a 2-triangle ground plane;
    roughness 0.05 -> 1 along x, metallic 0 -> 1 along y, base colour uniform in
    [0.2, 0.9]^3 from the seed; 512x256 RGB32F sky with a 5e3 sun disk and two
    point lights.  Float sky texels are physical, so both HDRI intensity
    multipliers are 1 (the reference default 350 scales 8-bit skies)."""
    rng = np.random.default_rng(seed)
    base = rng.uniform(0.2, 0.9, size=(49, 3)).astype(np.float32)
    sphere = uv_sphere(0.45, segments, rings)
    ground = quad((-14, 0, -14), (-14, 0, 14), (14, 0, 14), (14, 0, -14), (0, 1, 0))
    ground_mesh = MeshData(ground[0], ground[1],
                           uv0=np.array([[[0, 0], [0, 1], [1, 1]], [[0, 0], [1, 1], [1, 0]]], dtype=np.float32))
    meshes = [sphere, ground_mesh]
    materials, instances = [], []
    for j in range(7):  # metallic along y
        for i in range(7):  # roughness along x
            k = j * 7 + i
            materials.append(MaterialData(base_color=(float(base[k, 0]), float(base[k, 1]), float(base[k, 2]), 1.0),
                                          metallic=j / 6.0, roughness=0.05 + 0.95 * i / 6.0))
            instances.append(InstanceData(0, k, translate((i - 3) * 1.1, 0.55 + j * 1.1, 0.0)))
    materials.append(MaterialData(base_color=(0.5, 0.5, 0.5, 1.0), metallic=0.0, roughness=0.8))
    instances.append(InstanceData(1, 49))
    sky = TextureData(rgb32f=sky_texture(), filter=A.MT_FILTER_LINEAR)
    col = np.float32([1.0, 0.95, 0.9]) * np.float32(150.0)
    lights = [LightData(position=(-5.0, 9.0, 6.0), color=tuple(col), point_size=0.1),
              LightData(position=(6.0, 7.0, 5.0), color=tuple(np.float32([0.9, 0.95, 1.0]) * np.float32(120.0)),
                        point_size=0.1)]
    cam = CameraData(type=0, cam_to_world=translate(0.0, 3.8, 11.0), yfov=math.radians(45.0), aspect=16.0 / 9.0)
    scene = SceneData(meshes, instances, materials, [sky], lights, cam, env=0)
    cfg = make_config(width=width, height=height, samples=samples, ev_exposure=0.0, hdri_primary_intensity=1.0,
                      hdri_secondary_intensity=1.0, seed=seed)
    return scene, cfg


def num_grad_texels(s: SceneData) -> int:
    """Length of the texel-gradient buffer: RGB32F textures used as a base
    colour, in texture order (the layout mt_render_grad writes)."""
    used = {m.base_tex for m in s.materials if m.base_tex >= 0}
    return sum(t.rgb32f.size for i, t in enumerate(s.textures) if i in used and t.rgb32f is not None)


def adjoint_scene(width=512, height=512, samples=64, seed=0, texture_size=512, segments=64, rings=32):
    """Inverse-materials scene: the 7x7 material grid at 512x512 with a
    texture_size^2 RGB32F albedo texture on the ground plane (the parameters
    are the 49 spheres' base colour, roughness and metallic, the ground's
    texels and the two lights' intensities)."""
    scene, cfg = material_grid(width=width, height=height, samples=samples, seed=seed, segments=segments,
                               rings=rings)
    rng = np.random.default_rng(seed + 7)
    t = np.arange(texture_size)
    X, Y = np.meshgrid(t, t)
    checker = ((X // (texture_size // 8) + Y // (texture_size // 8)) % 2).astype(np.float32)
    albedo = np.stack([0.3 + 0.4 * checker, 0.35 + 0.1 * rng.random((texture_size, texture_size)),
                       0.5 - 0.3 * checker], -1).astype(np.float32)
    scene.textures.append(TextureData(rgb32f=albedo, filter=A.MT_FILTER_NEAREST, scale=(6.0, 6.0)))
    ground = scene.materials[49]
    ground.base_tex = len(scene.textures) - 1
    ground.base_color = (1.0, 1.0, 1.0, 1.0)
    cfg.width, cfg.height = width, height
    scene.camera.aspect = width / height
    return scene, cfg


def _value_noise(n, cells, rng):
    g = rng.random((cells + 1, cells + 1))
    x = np.linspace(0, cells, n, endpoint=False)
    i = x.astype(int)
    f = x - i
    f = f * f * (3 - 2 * f)
    a = g[i][:, i]
    b = g[i + 1][:, i]
    c = g[i][:, i + 1]
    d = g[i + 1][:, i + 1]
    fy, fx = f[:, None], f[None, :]
    return (a * (1 - fy) + b * fy) * (1 - fx) + (c * (1 - fy) + d * fy) * fx


def fbm(n, seed, octaves=6):
    rng = np.random.default_rng(seed)
    h = np.zeros((n, n))
    amp, cells = 1.0, 4
    for _ in range(octaves):
        h += amp * _value_noise(n, cells, rng)
        amp *= 0.5
        cells *= 2
    return h


def large_scene(terrain_n=1024, num_spheres=50_000, tex_size=2048, width=1920, height=1080, samples=1024,
                seed=0, extent=100.0):
    """fBm heightfield (2 * (n-1)^2 triangles) plus num_spheres icospheres of 80
    triangles, each set merged into one mesh, with procedural base-colour and
    tangent-space normal maps on the terrain."""
    rng = np.random.default_rng(seed)
    h = fbm(terrain_n, seed) * (extent * 0.08)
    xs = np.linspace(-extent / 2, extent / 2, terrain_n)
    X, Z = np.meshgrid(xs, xs)
    P = np.stack([X, h, Z], -1)
    dx = np.gradient(h, xs, axis=1)
    dz = np.gradient(h, xs, axis=0)
    N = np.stack([-dx, np.ones_like(h), -dz], -1)
    N /= np.linalg.norm(N, axis=-1, keepdims=True)
    UV = np.stack([(X / extent + 0.5) * 8.0, (Z / extent + 0.5) * 8.0], -1)

    def grid_tris(G):
        a, b, c, d = G[:-1, :-1], G[1:, :-1], G[1:, 1:], G[:-1, 1:]
        t1 = np.stack([a, b, c], axis=2).reshape(-1, 3, G.shape[-1])
        t2 = np.stack([a, c, d], axis=2).reshape(-1, 3, G.shape[-1])
        return np.concatenate([t1, t2]).astype(np.float32)

    terrain = MeshData(grid_tris(P), grid_tris(N), grid_tris(UV))
    ico = icosphere(1)
    cx = rng.uniform(-extent * 0.48, extent * 0.48, num_spheres)
    cz = rng.uniform(-extent * 0.48, extent * 0.48, num_spheres)
    r = rng.uniform(0.2, 0.6, num_spheres)
    ix = np.clip(((cx + extent / 2) / extent * (terrain_n - 1)).round().astype(int), 0, terrain_n - 1)
    iz = np.clip(((cz + extent / 2) / extent * (terrain_n - 1)).round().astype(int), 0, terrain_n - 1)
    cy = h[iz, ix] + r
    centers = np.stack([cx, cy, cz], -1)
    spos = (ico[None] * r[:, None, None, None] + centers[:, None, None, :]).reshape(-1, 3, 3).astype(np.float32)
    snrm = np.broadcast_to(ico[None], (num_spheres,) + ico.shape).reshape(-1, 3, 3).astype(np.float32)
    spheres = MeshData(spos, snrm)

    t = np.arange(tex_size)
    TX, TY = np.meshgrid(t, t)
    checker = ((TX // (tex_size // 16) + TY // (tex_size // 16)) % 2).astype(np.float64)
    noise = _value_noise(tex_size, 32, np.random.default_rng(seed + 1))
    base = np.stack([0.35 + 0.3 * checker + 0.2 * noise, 0.45 + 0.15 * noise, 0.25 + 0.2 * checker], -1)
    base_rgb8 = np.clip(base * 255.0, 0, 255).astype(np.uint8)
    hgt = _value_noise(tex_size, 64, np.random.default_rng(seed + 2))
    gy, gx = np.gradient(hgt)
    nm = np.stack([-gx * 20.0, -gy * 20.0, np.ones_like(hgt)], -1)
    nm /= np.linalg.norm(nm, axis=-1, keepdims=True)
    nrm_rgb8 = np.clip((nm * 0.5 + 0.5) * 255.0, 0, 255).astype(np.uint8)
    textures = [TextureData(rgb8=base_rgb8, filter=A.MT_FILTER_LINEAR),
                TextureData(rgb8=nrm_rgb8, filter=A.MT_FILTER_LINEAR),
                TextureData(rgb32f=sky_texture(), filter=A.MT_FILTER_LINEAR)]
    materials = [MaterialData(base_color=(1, 1, 1, 1), metallic=0.0, roughness=0.9, base_tex=0, normal_tex=1),
                 MaterialData(base_color=(0.8, 0.3, 0.2, 1), metallic=0.3, roughness=0.4)]
    instances = [InstanceData(0, 0), InstanceData(1, 1)]
    lights = [LightData(position=(0.0, extent * 0.4, 0.0), color=tuple(np.float32([1, 1, 1]) * np.float32(4000.0)),
                        point_size=0.5)]
    cam = CameraData(type=0, cam_to_world=_look_from(np.array([0.0, extent * 0.12, extent * 0.45]), -0.25),
                     yfov=math.radians(50.0), aspect=width / height)
    scene = SceneData([terrain, spheres], instances, materials, textures, lights, cam, env=2)
    cfg = make_config(width=width, height=height, samples=samples, ev_exposure=0.0, hdri_primary_intensity=1.0,
                      hdri_secondary_intensity=1.0, seed=seed)
    return scene, cfg


def _look_from(pos, pitch):
    c, s = math.cos(pitch), math.sin(pitch)
    m = np.eye(4, dtype=np.float32)
    m[1, 1], m[1, 2], m[2, 1], m[2, 2] = c, -s, s, c
    m[:3, 3] = pos
    return m


def scene_bounds(s: SceneData):
    lo = np.full(3, np.inf)
    hi = np.full(3, -np.inf)
    for it in s.instances:
        p = s.meshes[it.mesh].positions.reshape(-1, 3).astype(np.float64)
        p = p @ it.transform[:3, :3].T.astype(np.float64) + it.transform[:3, 3]
        lo = np.minimum(lo, p.min(0))
        hi = np.maximum(hi, p.max(0))
    return lo, hi


def incoherent_rays(lo, hi, n, seed=0, tmax=None) -> np.ndarray:
    """n rays as an (n, 8) float32 array in mt_ray layout: origins uniform in
    the box [lo, hi], directions uniform on the unit sphere."""
    rng = np.random.default_rng(seed)
    o = rng.uniform(lo, hi, size=(n, 3))
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = np.zeros((n, 8), dtype=np.float32)
    r[:, 0:3] = o
    r[:, 3] = np.float32(np.finfo(np.float32).max) if tmax is None else tmax
    r[:, 4:7] = d
    return r
