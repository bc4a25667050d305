"""The reference's own glTF test scenes (cornell box with an area light,
material spheres with a PNG checkerboard texture, the orthographic light-creep
scene), loaded by mitrace_gb300.gltf and committed as tests/golden/*.npz, run
end to end through the C ABI: counter-RNG renders match the oracle (99% of
pixels within 1e-4 + 1e-3 relative), with each scene's own exposure."""
from pathlib import Path

import numpy as np
import pytest

import mitrace_gb300 as mt
from oracle import oracle_py as orc
from tests.golden.scene_npz import load_scene

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.mark.parametrize("name", ["cornell_box", "material_spheres", "light_creep"])
def test_fixture_render_matches_oracle(name):
    scene, cfg, _ = load_scene(GOLDEN / f"{name}.npz")
    cfg.width, cfg.height, cfg.samples = 64, 64 if name != "light_creep" else 36, 16
    with mt.Tracer(scene, cfg) as tr:
        tr.StartRender()
        img = tr.WaitForRender().copy()
    ref, _, _ = orc.OracleScene(mt.PackedScene(scene), cfg).render(orc.RNG_COUNTER)
    assert img.max() > 0.01
    diff = np.abs(img - ref)
    ok = np.all(diff <= 1e-4 + 1e-3 * np.abs(ref), axis=-1)
    assert ok.mean() >= 0.99, f"{name}: {ok.mean():.4f}; max diff {diff.max():.3g}"
