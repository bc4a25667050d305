"""The C++ shim (include/mitrace/Tracer.hpp) compiles against the C ABI with a
plain C++ compiler, and on a GPU renders through it end to end."""
import subprocess
from pathlib import Path

import pytest

from mitrace_gb300 import _abi as A

ROOT = Path(__file__).resolve().parent.parent
SRC = ROOT / "tests" / "cpp" / "shim_box_room.cpp"


def build(tmp_path):
    exe = tmp_path / "shim_box_room"
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-I", str(ROOT / "include"), str(SRC), "-o",
                    str(exe), str(A.LIB_PATH), f"-Wl,-rpath,{A.LIB_PATH.parent}", "-pthread"], check=True)
    return exe


def test_shim_compiles(tmp_path):
    assert build(tmp_path).exists()


@pytest.mark.gpu
def test_shim_renders(tmp_path):
    out = subprocess.run([str(build(tmp_path)), str(tmp_path / "img")], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    f = out.stdout.split()
    assert f[0] == "ok"
    r, g, b = map(float, f[1:4])
    rays, samples, progress = int(f[4]), int(f[5]), float(f[6])
    assert samples == 64 * 64 * 16 and rays > samples and progress == 1.0
    assert 0.05 < r < 1.0 and abs(r - g) < 1e-3
    from mitrace_gb300 import gltf

    png = gltf.decode_png((tmp_path / "img.png").read_bytes())
    assert png.shape == (64, 64, 3) and abs(png[..., 0].mean() / 255.0 - r) < 0.01
    assert (tmp_path / "img.hdr").stat().st_size > 64 * 64 * 4
