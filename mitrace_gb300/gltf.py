"""glTF 2.0 (.gltf + .bin) loader into the boundary format, restating what
MiTrace's loader and scene conversion keep (src/Loader/GLTF.cpp,
src/Scene/Scene.cpp:12-59, Mesh.cpp:24-41, Light.hpp:36-56, Texture.cpp:17-33):

* meshes: every primitive of every node mesh becomes one instance with the
  node's world transform (parent * T * R * S, or the node matrix); POSITION and
  NORMAL are required, TEXCOORD_0 optional, indices (u16/u32) de-index the
  attributes (Mesh.cpp:9-31); accessors are read tightly packed (byteStride is
  ignored, GLTF.cpp:150-158), FLOAT attributes only; mode must be triangles;
* materials: pbrMetallicRoughness factors and textures, emissive factor times
  KHR_materials_emissive_strength, and ``normalScale`` / ``occlusionStrength``
  read from the material object itself (GLTF.cpp:476-483), not from the
  texture-info objects; a material without pbrMetallicRoughness is the default
  material; each instance gets its own material (Scene.cpp:38-41);
* textures: images by URI, RGB8 (alpha dropped), the sampler's minFilter
  (9728/9984/9985 nearest, else linear; linear without a sampler),
  KHR_texture_transform offset and scale (rotation and texCoord rejected);
* lights: KHR_lights_punctual point / spot / directional and
  EXT_light_attributes area lights on nodes; position = world transform
  column 3, colour = colour * intensity, spot cone cosines, direction =
  quat_cast(mat3(transform)) applied to (0, 0, -1);
* camera: the scene's cameras in node order, ``camera_index`` chosen (the
  first when out of range), yfov / aspectRatio or xmag / ymag;
* EXT_sky is parsed by the reference but Scene::Scene never copies the
  environment texture, so it is not used here either.

PNG images are decoded here (zlib, non-interlaced, 8/16-bit, all colour
types); JPEG needs a decoder this package does not have and raises.
"""
from __future__ import annotations

import json
import math
import struct
import zlib
from pathlib import Path
from typing import Dict, List, Optional, Tuple

import numpy as np

from . import _types as A
from .scenes import CameraData, InstanceData, LightData, MaterialData, MeshData, SceneData, TextureData, make_config

_F = np.float32


class GLTFError(RuntimeError):
    pass


# ----------------------------------------------------------------------------
# PNG (RFC 2083) -> RGB8, the result stbi_load(..., 3) gives
# ----------------------------------------------------------------------------
def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    if pa <= pb and pa <= pc:
        return a
    return b if pb <= pc else c


def decode_png(data: bytes) -> np.ndarray:
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise GLTFError("not a PNG file")
    pos, idat, palette, trns = 8, [], None, None
    w = h = depth = ctype = interlace = None
    while pos < len(data):
        n, kind = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + n]
        pos += 12 + n
        if kind == b"IHDR":
            w, h, depth, ctype, _, _, interlace = struct.unpack(">IIBBBBB", body)
        elif kind == b"PLTE":
            palette = np.frombuffer(body, np.uint8).reshape(-1, 3)
        elif kind == b"IDAT":
            idat.append(body)
        elif kind == b"IEND":
            break
    if w is None or interlace:
        raise GLTFError("interlaced or malformed PNG")
    channels = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    bits = channels * depth
    stride = (w * bits + 7) // 8
    bpp = max(1, bits // 8)
    raw = zlib.decompress(b"".join(idat))
    out = np.zeros((h, stride), np.uint8)
    prev = np.zeros(stride, np.int32)
    for y in range(h):
        f = raw[y * (stride + 1)]
        line = np.frombuffer(raw, np.uint8, stride, y * (stride + 1) + 1).astype(np.int32)
        if f == 0:
            cur = line
        elif f == 2:
            cur = (line + prev) & 0xFF
        else:
            cur = line.copy()
            for i in range(stride):
                a = cur[i - bpp] if i >= bpp else 0
                b = prev[i]
                c = prev[i - bpp] if i >= bpp else 0
                if f == 1:
                    cur[i] = (cur[i] + a) & 0xFF
                elif f == 3:
                    cur[i] = (cur[i] + ((a + b) >> 1)) & 0xFF
                elif f == 4:
                    cur[i] = (cur[i] + _paeth(a, b, c)) & 0xFF
                else:
                    raise GLTFError(f"bad PNG filter {f}")
        out[y] = cur
        prev = cur
    if depth == 16:
        px = out.reshape(h, w, channels * 2)[:, :, 0::2]  # high bytes
    elif depth == 8:
        px = out.reshape(h, w, channels)
    else:  # 1, 2, 4-bit grey or palette
        bitsarr = np.unpackbits(out, axis=1)[:, : w * depth].reshape(h, w, depth)
        px = np.zeros((h, w), np.int32)
        for k in range(depth):
            px = (px << 1) | bitsarr[:, :, k]
        if ctype == 0:
            px = (px * (255 // ((1 << depth) - 1))).astype(np.uint8)
        px = px[..., None].astype(np.uint8)
    if ctype == 3:
        if palette is None:
            raise GLTFError("palette PNG without PLTE")
        return palette[px[..., 0]].copy()
    if channels <= 2:
        return np.repeat(px[..., :1], 3, axis=2).copy()
    return px[..., :3].copy()


def load_image(path: Path) -> np.ndarray:
    data = path.read_bytes()
    if data[:8] == b"\x89PNG\r\n\x1a\n":
        return decode_png(data)
    raise GLTFError(f"{path.name}: only PNG images can be decoded here")


# ----------------------------------------------------------------------------
# GLM-convention transforms (float32)
# ----------------------------------------------------------------------------
def _quat_to_mat3(q) -> np.ndarray:
    """mat3_cast of (x, y, z, w) as a math (row-major) matrix."""
    x, y, z, w = (_F(v) for v in q)
    xx, yy, zz = x * x, y * y, z * z
    xz, xy, yz = x * z, x * y, y * z
    wx, wy, wz = w * x, w * y, w * z
    one, two = _F(1), _F(2)
    return np.array([[one - two * (yy + zz), two * (xy - wz), two * (xz + wy)],
                     [two * (xy + wz), one - two * (xx + zz), two * (yz - wx)],
                     [two * (xz - wy), two * (yz + wx), one - two * (xx + yy)]], _F)


def _quat_from_mat3(m: np.ndarray):
    """quat_cast (largest-component method of Shepperd / Shoemake); m is math
    row-major, so m[r][c] is GLM's m[c][r]."""
    g = lambda c, r: _F(m[r][c])  # noqa: E731  GLM column-major accessor
    four = [g(0, 0) - g(1, 1) - g(2, 2), g(1, 1) - g(0, 0) - g(2, 2), g(2, 2) - g(0, 0) - g(1, 1),
            g(0, 0) + g(1, 1) + g(2, 2)]  # x, y, z, w
    idx = 3
    big = four[3]
    for k in range(3):
        if four[k] > big:
            big, idx = four[k], k
    bv = _F(math.sqrt(float(big + _F(1)))) * _F(0.5)
    mult = _F(0.25) / bv
    if idx == 3:
        return ((g(1, 2) - g(2, 1)) * mult, (g(2, 0) - g(0, 2)) * mult, (g(0, 1) - g(1, 0)) * mult, bv)
    if idx == 0:
        return (bv, (g(0, 1) + g(1, 0)) * mult, (g(2, 0) + g(0, 2)) * mult, (g(1, 2) - g(2, 1)) * mult)
    if idx == 1:
        return ((g(0, 1) + g(1, 0)) * mult, bv, (g(1, 2) + g(2, 1)) * mult, (g(2, 0) - g(0, 2)) * mult)
    return ((g(2, 0) + g(0, 2)) * mult, (g(1, 2) + g(2, 1)) * mult, bv, (g(0, 1) - g(1, 0)) * mult)


def _quat_rotate(q, v) -> np.ndarray:
    """q * v as GLM computes it: v + 2 (w (u x v) + u x (u x v))."""
    u = np.array(q[:3], _F)
    w = _F(q[3])
    v = np.asarray(v, _F)
    uv = np.cross(u, v).astype(_F)
    uuv = np.cross(u, uv).astype(_F)
    return (v + ((uv * w) + uuv) * _F(2)).astype(_F)


def node_transform(node: dict) -> np.ndarray:
    """GLTF::ComputeNodeTransform (GLTF.cpp:265-292), math row-major."""
    if "matrix" in node:
        return np.array(node["matrix"], _F).reshape(4, 4).T.copy()  # column-major storage
    t = np.eye(4, dtype=_F)
    if "translation" in node:
        t[:3, 3] = np.array(node["translation"], _F)
    if "rotation" in node:
        r = np.eye(4, dtype=_F)
        r[:3, :3] = _quat_to_mat3(node["rotation"])
        t = (t @ r).astype(_F)
    if "scale" in node:
        t[:, :3] = t[:, :3] * np.array(node["scale"], _F)[None, :]
    return t


# ----------------------------------------------------------------------------
# Loader
# ----------------------------------------------------------------------------
_ACCESSOR_TYPES = {"SCALAR": 1, "VEC2": 2, "VEC3": 3, "VEC4": 4}
_COMPONENTS = {5126: np.float32, 5123: np.uint16, 5125: np.uint32}
_NEAREST = {9728, 9984, 9985}


class GLTF:
    def __init__(self, path):
        self.path = Path(path)
        self.base = self.path.parent
        try:
            self.j = json.loads(self.path.read_text())
        except Exception as e:  # noqa: BLE001
            raise GLTFError(f"Failed to load GLTF file '{self.path}': {e}") from e
        self._buffers: Dict[int, bytes] = {}
        self._meshes: Dict[Tuple[int, int], int] = {}
        self._textures: Dict[tuple, int] = {}
        self._images: Dict[str, np.ndarray] = {}
        self.scene = SceneData(meshes=[], instances=[], materials=[])

    # -- buffers and accessors (GLTF.cpp:42-171)
    def buffer(self, i: int) -> bytes:
        if i not in self._buffers:
            b = self.j["buffers"][i]
            uri = b["uri"]
            if uri.startswith("data:"):
                raise GLTFError("Data URI buffers are not supported")
            data = (self.base / uri).read_bytes()
            n = int(b["byteLength"])
            if len(data) < n:
                raise GLTFError(f"Failed to read buffer file: {uri}")
            self._buffers[i] = data[:n]
        return self._buffers[i]

    def accessor(self, i: int, want_type: Optional[str] = None, want_comp=None) -> np.ndarray:
        a = self.j["accessors"][i]
        kind = a["type"]
        if kind not in _ACCESSOR_TYPES:
            raise GLTFError("Unsupported attribute type for loading data")
        if a["componentType"] not in _COMPONENTS:
            raise GLTFError("Unsupported component type for attribute data")
        dt = _COMPONENTS[a["componentType"]]
        if want_type and (kind != want_type or (want_comp is not None and dt not in want_comp)):
            raise GLTFError("Attribute type does not match expected type")
        bv = self.j["bufferViews"][a["bufferView"]]
        data = self.buffer(bv["buffer"])
        off = int(a.get("byteOffset", 0)) + int(bv.get("byteOffset", 0))
        n = _ACCESSOR_TYPES[kind]
        arr = np.frombuffer(data, dtype=np.dtype(dt).newbyteorder("<"), count=int(a["count"]) * n, offset=off)
        return arr.reshape(int(a["count"]), n) if n > 1 else arr.copy()

    # -- meshes (GLTF.cpp:294-406, Mesh.cpp:9-31)
    def mesh(self, mi: int, pi: int) -> int:
        key = (mi, pi)
        if key in self._meshes:
            return self._meshes[key]
        prim = self.j["meshes"][mi]["primitives"][pi]
        if "attributes" not in prim or "indices" not in prim:
            raise GLTFError("Invalid GLTF primitive data: missing attributes or indices")
        if prim.get("mode", 4) != 4:
            raise GLTFError("Only triangle primitives (mode 4) are supported")
        attr = prim["attributes"]
        if "POSITION" not in attr or "NORMAL" not in attr:
            raise GLTFError("POSITION and NORMAL attributes are required")
        idx = self.accessor(prim["indices"], "SCALAR", (np.uint16, np.uint32)).astype(np.int64)
        pos = self.accessor(attr["POSITION"], "VEC3", (np.float32,)).astype(_F)
        nrm = self.accessor(attr["NORMAL"], "VEC3", (np.float32,)).astype(_F)
        uv = self.accessor(attr["TEXCOORD_0"], "VEC2", (np.float32,)).astype(_F) if "TEXCOORD_0" in attr else None
        if idx.size % 3:
            raise GLTFError("index count is not a multiple of 3")
        t = idx.size // 3
        m = MeshData(positions=np.ascontiguousarray(pos[idx].reshape(t, 3, 3)),
                     normals=np.ascontiguousarray(nrm[idx].reshape(t, 3, 3)),
                     uv0=np.ascontiguousarray(uv[idx].reshape(t, 3, 2)) if uv is not None else None)
        self.scene.meshes.append(m)
        self._meshes[key] = len(self.scene.meshes) - 1
        return self._meshes[key]

    # -- textures (GLTF.cpp:208-262, Texture.cpp:17-33)
    def texture_info(self, info: dict) -> int:
        if info.get("texCoord", 0) != 0:
            raise GLTFError("Only TEXCOORD_0 is supported for texture info")
        tex = self.j["textures"][info["index"]]
        filt = A.MT_FILTER_LINEAR
        if "sampler" in tex:
            mf = self.j["samplers"][tex["sampler"]].get("minFilter", 9729)
            if mf not in _NEAREST | {9729, 9986, 9987}:
                raise GLTFError("Unsupported filter mode in texture sampler")
            filt = A.MT_FILTER_NEAREST if mf in _NEAREST else A.MT_FILTER_LINEAR
        offset, scale = (0.0, 0.0), (1.0, 1.0)
        tt = info.get("extensions", {}).get("KHR_texture_transform")
        if tt is not None:
            if "rotation" in tt:
                raise GLTFError("KHR_texture_transform rotation is not supported")
            if "texCoord" in tt:
                raise GLTFError("KHR_texture_transform texCoord override is not supported")
            offset = tuple(float(v) for v in tt.get("offset", offset))
            scale = tuple(float(v) for v in tt.get("scale", scale))
        img = self.j["images"][tex["source"]]
        if "uri" not in img:
            raise GLTFError("Only URI-based images are supported")
        path = str((self.base / img["uri"]).resolve())
        key = (path, filt, offset, scale)
        if key not in self._textures:
            if path not in self._images:
                self._images[path] = load_image(Path(path))
            self.scene.textures.append(TextureData(rgb8=self._images[path], filter=filt, offset=offset, scale=scale))
            self._textures[key] = len(self.scene.textures) - 1
        return self._textures[key]

    # -- materials (GLTF.cpp:434-500, Material.hpp:63-77)
    def material(self, prim: dict) -> MaterialData:
        if "material" not in prim:
            return MaterialData()
        md = self.j["materials"][prim["material"]]
        if "pbrMetallicRoughness" not in md:
            return MaterialData()
        pbr = md["pbrMetallicRoughness"]
        m = MaterialData()
        em = np.array(md.get("emissiveFactor", [0.0, 0.0, 0.0]), _F)
        strength = md.get("extensions", {}).get("KHR_materials_emissive_strength")
        if strength is not None:
            em = em * _F(strength.get("emissiveStrength", 1.0))
        m.emissive = tuple(float(v) for v in em)
        m.base_color = tuple(float(v) for v in pbr.get("baseColorFactor", [1.0, 1.0, 1.0, 1.0]))
        m.metallic = float(pbr.get("metallicFactor", 1.0))
        m.roughness = float(pbr.get("roughnessFactor", 1.0))
        if "emissiveTexture" in md:
            m.emissive_tex = self.texture_info(md["emissiveTexture"])
        if "baseColorTexture" in pbr:
            m.base_tex = self.texture_info(pbr["baseColorTexture"])
        if "metallicRoughnessTexture" in pbr:
            m.mr_tex = self.texture_info(pbr["metallicRoughnessTexture"])
        if "normalTexture" in md:
            m.normal_tex = self.texture_info(md["normalTexture"])
        m.normal_scale = float(md.get("normalScale", 1.0))
        if "occlusionTexture" in md:
            m.occlusion_tex = self.texture_info(md["occlusionTexture"])
        m.occlusion_strength = float(md.get("occlusionStrength", 1.0))
        if md.get("alphaMode", "OPAQUE") not in ("OPAQUE", "MASK", "BLEND"):
            raise GLTFError("Unsupported alpha mode in material")
        return m

    # -- lights (GLTF.cpp:555-690, Light.hpp:36-56)
    def light(self, ld: dict, kind: str, world: np.ndarray) -> LightData:
        color = np.array(ld.get("color", [1.0, 1.0, 1.0]), _F) * _F(ld.get("intensity", 1.0))
        types = {"point": A.MT_LIGHT_POINT, "directional": A.MT_LIGHT_DIRECTIONAL, "spot": A.MT_LIGHT_SPOT,
                 "area": A.MT_LIGHT_AREA}
        if kind not in types:
            raise GLTFError("Unsupported light type in GLTF")
        L = LightData(type=types[kind], position=tuple(float(v) for v in world[:3, 3]),
                      color=tuple(float(v) for v in color))
        inner, outer = 0.0, 0.0
        if kind == "point":
            L.point_size = float(ld.get("size", 0.1))
        elif kind == "spot":
            L.point_size = float(ld.get("size", 0.0))
            inner = float(ld["spot"].get("innerConeAngle", 0.0))
            outer = float(ld["spot"].get("outerConeAngle", math.pi / 4))
        elif kind == "area":
            shape = ld.get("shape")
            if shape is None:
                raise GLTFError("Area light missing 'shape' property")
            if shape not in ("rectangle", "disc"):
                raise GLTFError(f"Unsupported area light shape: {shape}")
            L.point_size = 0.1  # Loader::Light's default; area lights shade as points (Tracer.cpp:295-297)
        else:
            L.point_size = 0.1  # Loader::Light's default (Types.hpp:97)
        L.inner_cos = float(np.cos(_F(inner)))
        L.outer_cos = float(np.cos(_F(outer)))
        if kind in ("directional", "spot"):
            q = _quat_from_mat3(world[:3, :3])
            L.direction = tuple(float(v) for v in _quat_rotate(q, (0.0, 0.0, -1.0)))
        return L

    # -- node walk (GLTF.cpp:692-880)
    def walk(self, ni: int, parent: np.ndarray, cameras: list):
        node = self.j["nodes"][ni]
        world = (parent @ node_transform(node)).astype(_F)
        if "mesh" in node:
            mi = node["mesh"]
            for pi, prim in enumerate(self.j["meshes"][mi]["primitives"]):
                mesh_id = self.mesh(mi, pi)
                self.scene.materials.append(self.material(prim))
                self.scene.instances.append(InstanceData(mesh=mesh_id, material=len(self.scene.materials) - 1,
                                                         transform=world.copy()))
        ext = node.get("extensions", {})
        if "KHR_lights_punctual" in ext:
            li = ext["KHR_lights_punctual"]["light"]
            ld = self.j["extensions"]["KHR_lights_punctual"]["lights"][li]
            self.scene.lights.append(self.light(ld, ld["type"], world))
        if "EXT_light_attributes" in ext and "areaLight" in ext["EXT_light_attributes"]:
            ai = ext["EXT_light_attributes"]["areaLight"]
            ld = self.j["extensions"]["EXT_light_attributes"]["areaLights"][ai]
            self.scene.lights.append(self.light(ld, "area", world))
        if "camera" in node:
            cd = self.j["cameras"][node["camera"]]
            if cd["type"] == "perspective":
                p = cd["perspective"]
                cam = CameraData(type=0, cam_to_world=world.copy(), yfov=float(p["yfov"]),
                                 aspect=float(p.get("aspectRatio", 1.0)))
            elif cd["type"] == "orthographic":
                o = cd["orthographic"]
                cam = CameraData(type=1, cam_to_world=world.copy(), yfov=0.0,
                                 aspect=float(_F(o["xmag"]) / _F(o["ymag"])), ortho=(float(o["xmag"]), float(o["ymag"])))
            else:
                raise GLTFError("Unsupported camera type in GLTF")
            cameras.append(cam)
        for c in node.get("children", []):
            self.walk(c, world, cameras)

    def load(self, scene_index: int = 0, camera_index: int = 0) -> SceneData:
        cameras: List[CameraData] = []
        for ni in self.j["scenes"][scene_index]["nodes"]:
            self.walk(ni, np.eye(4, dtype=_F), cameras)
        if not cameras:
            raise GLTFError("No camera found in the scene")
        self.scene.camera = cameras[camera_index if camera_index < len(cameras) else 0]
        return self.scene


def load_gltf(path, scene_index: int = 0, camera_index: int = 0) -> SceneData:
    return GLTF(path).load(scene_index, camera_index)


def parse_render_params(text: str, **overrides):
    """The CLI flags of a fixture's render_params.txt -> mt_config."""
    names = {"--width": "width", "--height": "height", "--samples": "samples", "--ev-exposure": "ev_exposure",
             "--bounces": "bounces", "--firefly-threshold": "firefly_threshold",
             "--terminate-energy": "terminate_energy"}
    tok = text.split()
    kw = {}
    for i, t in enumerate(tok):
        if t in names and i + 1 < len(tok):
            v = tok[i + 1]
            kw[names[t]] = float(v) if "." in v or names[t] in ("ev_exposure", "firefly_threshold",
                                                                 "terminate_energy") else int(v)
    kw.update(overrides)
    return make_config(**kw)
