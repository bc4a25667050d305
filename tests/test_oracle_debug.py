"""Known answers for the oracle's debug render modes (ProcessDebugRay,
src/Tracer/Tracer.cpp:366-488; heatmap post-processing 650-716): the box room's
albedo, metallic/roughness and geometric-normal images take the scene's exact
values inside faces, and heatmap images end at the ramp's ends."""
import numpy as np

import mitrace_gb300 as mt
from oracle import oracle_py as orc


def oracle_image(mode, samples=4, **kw):
    scene, cfg = mt.box_room(width=40, height=40, samples=samples, seed=1, **kw)
    cfg.debug_mode = mode
    img, _, _ = orc.OracleScene(mt.PackedScene(scene), cfg).render(orc.RNG_COUNTER)
    return scene, img


def interior(img, value):
    return np.all(np.abs(img - np.asarray(value, np.float32)) == 0, axis=-1)


def test_albedo_is_the_remapped_base_colour():
    scene, img = oracle_image(5)
    colours = [np.float32(m.base_color[:3]) * np.float32(0.96) + np.float32(0.04) for m in scene.materials]
    hit = np.zeros(img.shape[:2], bool)
    for c in colours:
        hit |= interior(img, c)
    assert hit.mean() > 0.8  # all but the pixels whose samples straddle two materials


def test_metallic_roughness_channels():
    scene, img = oracle_image(6)
    m = scene.materials[0]
    assert np.all(img[..., 0] == 0)
    assert interior(img, (0.0, m.metallic, m.roughness)).mean() > 0.8


def test_geometric_normals_of_axis_aligned_faces():
    _, img = oracle_image(7)
    axis = [(0.5, 1.0, 0.5), (0.5, 0.0, 0.5), (1.0, 0.5, 0.5), (0.0, 0.5, 0.5), (0.5, 0.5, 1.0), (0.5, 0.5, 0.0)]
    ok = np.zeros(img.shape[:2], bool)
    for a in axis:
        ok |= np.all(np.abs(img - np.float32(a)) < 1e-6, axis=-1)
    assert ok.mean() > 0.8


def test_heatmap_modes_span_the_ramp():
    _, img = oracle_image(4)  # total triangle tests
    red = np.all(img == np.float32([1, 0, 0]), axis=-1)
    assert red.any()
    assert np.all(img >= 0) and np.all(img <= 1)
    _, grey = oracle_image(16)  # depth, grey ramp
    assert np.allclose(grey[..., 0], grey[..., 1]) and grey.max() == 1.0
