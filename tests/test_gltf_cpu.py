"""The glTF loader (mitrace_gb300/gltf.py) and the committed fixtures made from
the reference's own test scenes (tests/golden/make_gltf_fixtures.py)."""
import math
import os
from pathlib import Path

import numpy as np
import pytest

import mitrace_gb300 as mt
from mitrace_gb300 import gltf
from oracle import oracle_py as orc
from tests.golden.scene_npz import load_scene

GOLDEN = Path(__file__).resolve().parent / "golden"
# a MiTrace checkout, when one is at hand: the fixtures are re-derived from it
REF = Path(os.environ["MITRACE_REFERENCE"]) if os.environ.get("MITRACE_REFERENCE") else None
NAMES = ["cornell_box", "material_spheres", "light_creep"]


def test_png_decoder_filters_and_colour_types():
    import struct
    import zlib

    rng = np.random.default_rng(0)
    img = rng.integers(0, 256, (5, 7, 4), dtype=np.uint8)

    def png(ctype, rows):
        def chunk(k, b):
            return struct.pack(">I", len(b)) + k + b + struct.pack(">I", zlib.crc32(k + b) & 0xffffffff)
        ch = {2: 3, 6: 4, 0: 1}[ctype]
        raw = b""
        prev = np.zeros(7 * ch, np.int32)
        for y, f in enumerate(rows):
            line = img[y, :, :ch].reshape(-1).astype(np.int32)
            if f == 0:
                enc = line
            elif f == 1:
                left = np.concatenate([np.zeros(ch, np.int32), line[:-ch]])
                enc = (line - left) & 0xFF
            elif f == 2:
                enc = (line - prev) & 0xFF
            elif f == 3:
                left = np.concatenate([np.zeros(ch, np.int32), line[:-ch]])
                enc = (line - ((left + prev) >> 1)) & 0xFF
            else:
                left = np.concatenate([np.zeros(ch, np.int32), line[:-ch]])
                upl = np.concatenate([np.zeros(ch, np.int32), prev[:-ch]])
                pr = np.array([gltf._paeth(a, b, c) for a, b, c in zip(left, prev, upl)], np.int32)
                enc = (line - pr) & 0xFF
            raw += bytes([f]) + bytes(enc.astype(np.uint8))
            prev = line
        return (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", 7, 5, 8, ctype, 0, 0, 0))
                + chunk(b"IDAT", zlib.compress(raw)) + chunk(b"IEND", b""))

    for ctype in (2, 6):
        out = gltf.decode_png(png(ctype, [0, 1, 2, 3, 4]))
        np.testing.assert_array_equal(out, img[:, :, :3])
    grey = gltf.decode_png(png(0, [4, 3, 2, 1, 0]))
    np.testing.assert_array_equal(grey, np.repeat(img[:, :, :1], 3, axis=2))


def test_quaternion_helpers():
    rng = np.random.default_rng(1)
    for _ in range(50):
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        m = gltf._quat_to_mat3(q)
        np.testing.assert_allclose(m @ m.T, np.eye(3), atol=1e-5)
        q2 = np.array(gltf._quat_from_mat3(m), np.float64)
        assert min(np.abs(q2 - q).max(), np.abs(q2 + q).max()) < 1e-5
        v = rng.normal(size=3)
        np.testing.assert_allclose(gltf._quat_rotate(q2, v), m @ v, atol=1e-4)


def test_node_transform_is_translate_rotate_scale():
    node = {"translation": [1, 2, 3], "rotation": [0, math.sin(0.25), 0, math.cos(0.25)], "scale": [2, 3, 4]}
    t = gltf.node_transform(node)
    r = gltf._quat_to_mat3(node["rotation"])
    expect = np.eye(4)
    expect[:3, :3] = r @ np.diag([2, 3, 4])
    expect[:3, 3] = [1, 2, 3]
    np.testing.assert_allclose(t, expect, atol=1e-6)
    m = np.arange(16, dtype=np.float32)
    np.testing.assert_array_equal(gltf.node_transform({"matrix": m.tolist()}), m.reshape(4, 4).T)


@pytest.mark.skipif(REF is None or not REF.exists(), reason="MITRACE_REFERENCE does not name a MiTrace checkout")
@pytest.mark.parametrize("name", NAMES)
def test_loader_reproduces_the_committed_fixture(name, tmp_path):
    from tests.golden.make_gltf_fixtures import FIXTURES
    from tests.golden.scene_npz import save_scene

    path = REF / FIXTURES[name]
    scene = gltf.load_gltf(path)
    cfg = gltf.parse_render_params((path.parent / "render_params.txt").read_text())
    save_scene(tmp_path / "x.npz", scene, cfg)
    a, ca, _ = load_scene(tmp_path / "x.npz")
    b, cb, _ = load_scene(GOLDEN / f"{name}.npz")
    assert mt.scenes.config_dict(ca) == mt.scenes.config_dict(cb)
    for ma, mb in zip(a.meshes, b.meshes):
        np.testing.assert_array_equal(ma.positions, mb.positions)
        np.testing.assert_array_equal(ma.normals, mb.normals)
    assert [l.__dict__ for l in a.lights] == [l.__dict__ for l in b.lights]


@pytest.mark.parametrize("name", NAMES)
def test_fixtures_render_on_the_oracle(name):
    scene, cfg, meta = load_scene(GOLDEN / f"{name}.npz")
    cfg.width, cfg.height, cfg.samples = 32, 32, 4
    scene.camera.aspect = scene.camera.aspect  # the fixture's own camera
    img, rays, samples = orc.OracleScene(mt.PackedScene(scene), cfg).render(orc.RNG_COUNTER)
    assert np.isfinite(img).all() and img.max() > 0.01
    assert samples == 32 * 32 * 4 and rays >= samples


def test_fixture_contents():
    s, c, _ = load_scene(GOLDEN / "cornell_box.npz")
    assert s.num_triangles == 42 and len(s.lights) == 1 and s.lights[0].type == mt._abi.MT_LIGHT_AREA
    assert (c.width, c.height, c.samples, c.ev_exposure) == (512, 512, 512, 6.0)
    s, c, _ = load_scene(GOLDEN / "material_spheres.npz")
    assert s.num_triangles == 7214 and len(s.textures) == 1 and s.textures[0].shape == (256, 256, 3)
    s, c, _ = load_scene(GOLDEN / "light_creep.npz")
    assert s.camera.type == 1 and s.num_triangles == 56
