"""Edge cases of the render path against the oracle (same counter RNG):
an empty scene (sky only, and black without a sky), a scene without lights,
spot / directional / area lights (the reference shades every non-spot light
as a point at its node position, Tracer.cpp:295-297), a 1x1 image at 1 spp
and 1 bounce, ragged batches and bands, the tiled path order at ragged
image edges, and a zero-spp config rejected."""
import ctypes as C

import numpy as np
import pytest

import mitrace_gb300 as mt
from mitrace_gb300 import _abi as A
from oracle import oracle_py as orc

from .helpers import small_grid

pytestmark = pytest.mark.gpu


def both(scene, cfg):
    with mt.Tracer(scene, cfg) as tr:
        tr.StartRender()
        img = tr.WaitForRender().copy()
        st = tr.GetStats()
    ref, rays, samples = orc.OracleScene(mt.PackedScene(scene), cfg).render(orc.RNG_COUNTER)
    return img, ref, st, rays, samples


def close(img, ref, frac=0.99):
    diff = np.abs(img - ref)
    ok = np.all(diff <= 1e-4 + 1e-3 * np.abs(ref), axis=-1)
    assert ok.mean() >= frac, (ok.mean(), diff.max())


def test_empty_scene_sky_and_black():
    grid, gcfg = small_grid(width=24, height=16, samples=4)
    scene = mt.SceneData(meshes=[], instances=[], materials=[], textures=grid.textures, lights=[],
                         camera=grid.camera, env=grid.env)
    img, ref, st, rays, samples = both(scene, gcfg)
    np.testing.assert_allclose(img, ref, rtol=1e-5, atol=1e-6)
    assert st.rays == rays == samples == 24 * 16 * 4  # one primary ray per sample, no shadow rays
    assert img.max() > 0
    scene.env = -1
    img, ref, *_ = both(scene, gcfg)
    assert np.all(img == 0) and np.all(ref == 0)


def test_scene_without_lights():
    scene, cfg = mt.box_room(width=32, height=32, samples=8, seed=4)
    scene.lights = []
    img, ref, *_ = both(scene, cfg)
    close(img, ref)


@pytest.mark.parametrize("kind", [A.MT_LIGHT_SPOT, A.MT_LIGHT_DIRECTIONAL, A.MT_LIGHT_AREA])
def test_light_types(kind):
    scene, cfg = mt.box_room(width=32, height=32, samples=8, seed=5)
    L = scene.lights[0]
    L.type = kind
    L.direction = (0.0, -1.0, 0.0)
    L.inner_cos, L.outer_cos = float(np.cos(0.3)), float(np.cos(0.6))
    img, ref, *_ = both(scene, cfg)
    close(img, ref)
    assert img.max() > 0.01


def test_single_pixel_single_sample_single_bounce():
    scene, cfg = mt.box_room(width=1, height=1, samples=1, seed=6)
    cfg.bounces = 1
    img, ref, st, rays, samples = both(scene, cfg)
    close(img, ref, frac=1.0)
    assert st.samples == samples == 1


def test_ragged_batches_and_bands(monkeypatch):
    scene, cfg = small_grid(width=37, height=23, samples=5, seed=8)
    monkeypatch.setenv("MT_BATCH_PATHS", "1021")  # batches that split pixels and samples unevenly
    monkeypatch.setenv("MT_SAMPLE_BUDGET_MB", "0")  # one image row per band
    img, ref, *_ = both(scene, cfg)
    close(img, ref)


def test_tiled_path_order_with_ragged_edges(monkeypatch):
    """One 37x23 band: four rows of whole 8x4 pixel tiles, the 5 columns right
    of them and the 3 rows below, in batches of 1021 paths that cut tiles and
    samples.  The image equals the oracle's, and bit for bit the one rendered
    in bands of one row (whose paths keep the row-major order)."""
    scene, cfg = small_grid(width=37, height=23, samples=5, seed=9)
    monkeypatch.setenv("MT_BATCH_PATHS", "1021")
    img, ref, st, rays, samples = both(scene, cfg)
    close(img, ref)
    assert st.samples == samples and st.rays == rays
    monkeypatch.setenv("MT_SAMPLE_BUDGET_MB", "0")  # one image row per band
    row_major, *_ = both(scene, cfg)
    np.testing.assert_array_equal(img, row_major)


def test_zero_samples_rejected():
    scene, _ = mt.box_room()
    cfg = mt.make_config(width=8, height=8, samples=0)
    ps = mt.PackedScene(scene)
    h = C.c_void_p()
    assert A.lib.mt_create(ps.ptr(), C.byref(cfg), C.byref(h)) == A.MT_ERR_INVALID
