"""bench.py's contract pieces that need no GPU: default arguments (N = 1, at
least 3 warm-up steps, the 1080p time-to-relMSE workload), the config dict both
arms print (identical by construction), and the CPU reference arm, which must
not load the product library."""
import importlib.util
import json
import subprocess
import sys

from tests.conftest import ROOT


def load_bench(monkeypatch, argv):
    spec = importlib.util.spec_from_file_location("bench_under_test", ROOT / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    monkeypatch.setattr(sys, "argv", ["bench.py", *argv])
    return mod, mod.parse()


def test_default_arguments(monkeypatch):
    bench, a = load_bench(monkeypatch, [])
    assert a.gpus == 1 and a.steps >= 1 and a.warmup >= 3
    assert a.impl == "ours"
    assert (a.width, a.height) == (1920, 1080)
    assert a.relmse_target == 0.01 and a.ref_spp == 16384


def test_both_arms_print_the_same_config(monkeypatch):
    bench, a = load_bench(monkeypatch, [])
    s1, c1 = bench.scene_and_config(a, a.spp, 0)
    s2, c2 = bench.scene_and_config(a, a.spp, 1234)
    assert bench.workload_config(a, s1, c1) == bench.workload_config(a, s2, c2)
    cfg = bench.workload_config(a, s1, c1)
    assert cfg["spp"] == a.spp and cfg["triangles"] == 49 * 4096 + 2
    json.dumps(cfg)


def test_reference_arm_loads_no_product_library(tmp_path):
    """A tiny run of the CPU arm (64x36, 2 spp) in a fresh process: it prints
    one JSON line with impl "reference" and never maps libmitrace_gb300.so."""
    code = (
        "import runpy, sys\n"
        "sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '0', '--width', '64',"
        " '--height', '36', '--spp', '2']\n"
        "try:\n"
        "    runpy.run_path(%r, run_name='__main__')\n"
        "finally:\n"
        "    maps = open('/proc/self/maps').read()\n"
        "    assert 'libmitrace_gb300' not in maps, 'product library mapped'\n" % str(ROOT / "bench.py")
    )
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "s" and line["higher_is_better"] is False
    assert line["config"]["spp"] == 2 and line["e2e"]["value"] == line["value"]
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
