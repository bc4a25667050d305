"""C ABI checks that need no GPU: the library loads, exports every function the
header declares, the ctypes mirror has the C layout, defaults match the
reference's Config.hpp, and argument errors come back as status codes."""
import ctypes as C
import re
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

import mitrace_gb300 as mt
from mitrace_gb300 import _abi as A

ROOT = Path(__file__).resolve().parent.parent
HEADERS = sorted((ROOT / "include").glob("*.h"))


def declared_functions():
    names = set()
    for h in HEADERS:
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:[\w\s\*]+?)\b(mt_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_every_declared_symbol_is_exported():
    names = declared_functions()
    assert len(names) >= 15
    lib = C.CDLL(str(A.LIB_PATH))
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # the ctypes mirror covers exactly the declared set
    assert sorted(p[0] for p in A.PROTOTYPES) == names


def test_abi_version():
    assert A.lib.mt_abi_version() == 1


C_LAYOUT = r"""
#include <stdio.h>
#include <stddef.h>
#include "mitrace_gpu.h"
#define S(T) printf(#T " %zu\n", sizeof(T));
#define O(T, f) printf(#T "." #f " %zu\n", offsetof(T, f));
int main(void) {
  S(mt_bvh_node) S(mt_mesh_desc) S(mt_texture_desc) S(mt_material_desc) S(mt_instance_desc)
  S(mt_light_desc) S(mt_camera_desc) S(mt_scene_desc) S(mt_config) S(mt_stats) S(mt_ray)
  S(mt_hit) S(mt_brdf_query) S(mt_brdf_result) S(mt_stage_profile) S(mt_profile) S(mt_grad_buffers) S(mt_nrc_config) S(mt_nrc_stats) S(mt_brdf_sample_query) S(mt_brdf_sample_result)
  O(mt_scene_desc, camera) O(mt_scene_desc, env_texture) O(mt_config, seed) O(mt_mesh_desc, bvh_indices)
  O(mt_texture_desc, filter) O(mt_light_desc, direction) O(mt_hit, tri_tests) O(mt_nrc_config, seed) O(mt_nrc_config, ema_decay) O(mt_nrc_config, end_at) O(mt_nrc_stats, train_loss) O(mt_grad_buffers, d_image)
  return 0;
}
"""


def test_ctypes_layout_matches_c_compiler(tmp_path):
    src = tmp_path / "layout.c"
    src.write_text(C_LAYOUT)
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    for line in filter(None, out):
        key, val = line.split()
        if "." in key:
            t, f = key.split(".")
            assert getattr(A, t).__dict__[f].offset == int(val), key
        else:
            assert C.sizeof(getattr(A, key)) == int(val), key
    assert C.sizeof(A.mt_ray) == 32 and C.sizeof(A.mt_hit) == 32 and C.sizeof(A.mt_bvh_node) == 32


def test_config_defaults_match_reference():
    c = mt.make_config()
    # src/CLI/Config.hpp:50-70
    assert (c.width, c.height, c.samples, c.bounces) == (1280, 720, 64, 5)
    assert c.ev_exposure == 8.0
    assert (c.hdri_primary_intensity, c.hdri_secondary_intensity, c.emission_base_intensity) == (350.0, 350.0, 1.0)
    assert (c.bvh_disable, c.bvh_max_triangles, c.bvh_max_depth) == (0, 32, 32)
    assert (c.firefly_enable, c.firefly_threshold) == (1, 6.0)
    assert abs(c.terminate_energy - 0.01) < 1e-9
    assert c.debug_mode == 0


def test_argument_errors_are_status_codes():
    h = C.c_void_p()
    assert A.lib.mt_create(None, None, C.byref(h)) == A.MT_ERR_INVALID
    assert h.value is None
    assert "required" in A.lib.mt_last_error().decode()
    cfg = mt.make_config(width=0)
    scene, _ = mt.box_room()
    ps = mt.PackedScene(scene)
    assert A.lib.mt_create(ps.ptr(), C.byref(cfg), C.byref(h)) == A.MT_ERR_INVALID
    for bad in (-1, 23):  # Config::DebugMode has 23 values
        cfg = mt.make_config(debug_mode=bad)
        assert A.lib.mt_create(ps.ptr(), C.byref(cfg), C.byref(h)) == A.MT_ERR_INVALID
    assert A.lib.mt_start(None) == A.MT_ERR_INVALID
    assert A.lib.mt_is_done(None) == 0
    assert A.lib.mt_brdf_batch(None, 4, None) == A.MT_ERR_INVALID
    assert A.lib.mt_resolve_batch(None, 4, 4, 1, 4.0, 0, None) == A.MT_ERR_INVALID
    one = np.zeros(3, np.float32)
    assert A.lib.mt_resolve_batch(one.ctypes.data, 1, 0, 1, 4.0, 0, one.ctypes.data) == A.MT_ERR_INVALID
    assert A.lib.mt_resolve_batch(one.ctypes.data, 1, 1, 1, 4.0, 99, one.ctypes.data) == A.MT_ERR_INVALID
    assert A.lib.mt_brdf_sample_batch(None, 4, None) == A.MT_ERR_INVALID
    assert A.lib.mt_update_materials(None, None, 0) == A.MT_ERR_INVALID
    assert A.lib.mt_update_lights(None, None, 0) == A.MT_ERR_INVALID
    assert A.lib.mt_update_texture(None, 0, None) == A.MT_ERR_INVALID
    assert A.lib.mt_write_png(None, None, 0, 0) == A.MT_ERR_INVALID


def test_create_without_gpu_fails_cleanly():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    scene, cfg = mt.box_room()
    with pytest.raises(mt.MTError) as e:
        mt.Tracer(scene, cfg)
    assert e.value.code == A.MT_ERR_CUDA


def test_packed_scene_round_trip():
    scene, cfg = mt.material_grid(width=64, height=36, samples=1)
    ps = mt.PackedScene(scene)
    d = ps.desc
    assert d.num_meshes == 2 and d.num_instances == 50 and d.num_materials == 50 and d.env_texture == 0
    assert d.meshes[0].num_triangles == 4096
    # column-major transform: translation in elements 12..14
    t = np.array(d.instances[8].transform[:])
    np.testing.assert_allclose(t[12:15], scene.instances[8].transform[:3, 3])
    assert d.textures[0].width == 512 and d.textures[0].height == 256


def test_python_config_defaults_equal_the_library_defaults():
    from mitrace_gb300 import _types

    a, b = A.mt_config(), _types.config_defaults(_types.mt_config())
    A.lib.mt_config_defaults(C.byref(a))
    assert bytes(a) == bytes(b)


def test_scene_generators_load_no_product_library():
    """The benchmark's CPU reference arm builds its scenes with
    mitrace_gb300.scenes; that import must not map libmitrace_gb300.so."""
    code = (
        "import sys; sys.path.insert(0, %r)\n"
        "import mitrace_gb300.scenes as S\n"
        "scene, cfg = S.material_grid(width=16, height=8, samples=1, segments=8, rings=4)\n"
        "S.PackedScene(scene)\n"
        "maps = open('/proc/self/maps').read()\n"
        "assert 'libmitrace_gb300' not in maps, 'product library mapped'\n"
        "print('ok')\n" % str(ROOT)
    )
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stderr
