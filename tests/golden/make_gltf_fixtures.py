"""Writes tests/golden/<name>.npz from the reference's glTF test scenes
(assets/tests/*/ of the MiTrace project) with mitrace_gb300.gltf, plus the
render settings of each scene's render_params.txt.  Run from the repository
root with the path of a MiTrace checkout (or set MITRACE_REFERENCE to it):

    python tests/golden/make_gltf_fixtures.py <path to the MiTrace checkout>

Scenes whose textures are JPEG (light_type_test, offset_scale_test,
normal_mapping_test) are skipped: no JPEG decoder is available here.
"""
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from mitrace_gb300 import gltf  # noqa: E402
from tests.golden.scene_npz import save_scene  # noqa: E402

FIXTURES = {
    "cornell_box": "assets/tests/cornell_box_test/cornell_box.gltf",
    "material_spheres": "assets/tests/material_spheres_test/material_spheres.gltf",
    "light_creep": "assets/tests/light_creep_test/light_creep_test.gltf",
}


def main(ref_root):
    ref_root = Path(ref_root)
    for name, rel in FIXTURES.items():
        path = ref_root / rel
        scene = gltf.load_gltf(path)
        cfg = gltf.parse_render_params((path.parent / "render_params.txt").read_text())
        save_scene(ROOT / "tests" / "golden" / f"{name}.npz", scene, cfg, meta={"source": rel})
        print(name, scene.num_triangles, "triangles", len(scene.lights), "lights")


if __name__ == "__main__":
    import os

    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("MITRACE_REFERENCE")
    if not root:
        sys.exit("usage: make_gltf_fixtures.py <MiTrace checkout>  (or set MITRACE_REFERENCE)")
    main(root)
