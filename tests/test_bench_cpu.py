"""bench.py's contract pieces that need no GPU: default arguments (N = 1, at
least 3 warm-up steps), the workload name of the default run, and the ncu
summary that the roofline's DRAM traffic is read from (it must name the same
workload and carry a per-ray figure, or the bench line would silently report
no traffic)."""
import importlib.util
import re
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
    assert (a.width, a.height, a.spp) == (1920, 1080, 256)


def test_traffic_summary_matches_default_workload(monkeypatch):
    bench, a = load_bench(monkeypatch, [])
    text = bench.TRAFFIC_FILE.read_text()
    w = re.findall(r"^traffic_workload: (\S+)$", text, re.M)
    b = re.findall(r"^traffic_bytes_per_extend_ray: ([0-9.]+)$", text, re.M)
    assert w == [bench.workload_name(a)], w
    assert len(b) == 1 and 0.0 < float(b[0]) < 1e4, b


def test_reference_arm_keeps_the_metric(monkeypatch):
    _, a = load_bench(monkeypatch, ["--impl", "reference", "--steps", "2", "--warmup", "3"])
    assert a.impl == "reference" and a.steps == 2 and a.warmup == 3
