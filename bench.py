#!/usr/bin/env python3
"""Benchmark of the path-tracing hot path on one GB300.

A step is one full render of the material-grid scene (7x7 spheres of 4096
triangles on a ground plane, float sky with a sun disk, 2 point lights) at
1920x1080 and 256 samples per pixel, through the C ABI.  The metric is the
reference's own throughput figure, Mrays/s, with rays counted the way
Tracer::GeneratePath / ProcessRayForward count them (one per extension ray,
one per shadow ray; src/Tracer/Tracer.cpp:146,319).

  value      device-resident: mt_render_device into a device image, CUDA-event
             time of each step on the launching stream, L2 flushed between steps
  e2e        host API: mt_create from host arrays (scene upload, BVH build),
             mt_start, mt_wait into a host image, mt_destroy; wall clock
  roofline   the traversal ("extend") kernel: algorithmic bytes per launch
             (64 B per inner-node expansion, 40 B per triangle test, 48 B per
             ray, counted by an untimed counting pass of the same render) over
             its CUDA-event launch time recorded inside the timed steps
  cpu_baseline  the CPU oracle (restatement of the reference, -Ofast, all host
             cores, reference tile queue) on a bounded band of rows

--impl reference times that CPU implementation alone (the reference itself
cannot be built here).  Under torchrun with N > 1 every rank renders its own
copy of the image ("replicas only": a render does not shard across GPUs in this
build) and rank 0 reports the aggregate.
"""
from __future__ import annotations

import argparse
import json
import re
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

PEAKS_FILE = ROOT / "MEASURED_PEAKS.json"
TRAFFIC_FILE = ROOT / "profiles" / "k_extend_material_grid.md"
FALLBACK_HBM_GBS = 6800.0


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--width", type=int, default=1920)
    p.add_argument("--height", type=int, default=1080)
    p.add_argument("--spp", type=int, default=256)
    p.add_argument("--e2e-steps", type=int, default=None)
    p.add_argument("--cpu-seconds", type=float, default=12.0, help="target length of the CPU baseline sample")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-microbench", action="store_true",
                   help="skip the 16M incoherent-ray closest/any-hit microbench on the large scene")
    p.add_argument("--microbench-rays", type=int, default=1 << 24)
    p.add_argument("--time-to-relmse", action="store_true",
                   help="instead of the throughput line: time to relMSE 0.01 against a high-spp reference")
    p.add_argument("--ref-spp", type=int, default=16384)
    p.add_argument("--relmse-target", type=float, default=0.01)
    p.add_argument("--no-nrc", action="store_true", help="time-to-relMSE: skip the radiance-cache leg")
    p.add_argument("--nrc-kernels-only", action="store_true",
                   help="only time the radiance cache's inference and training kernels")
    p.add_argument("--nrc-rows", type=int, default=1920 * 1080 * 4)
    p.add_argument("--nrc-warmup", type=int, default=0, help="training-only frames before the first cached frame")
    p.add_argument("--nrc-frames", type=int, default=48, help="cached frames at most")
    p.add_argument("--nrc-steps", type=int, default=None, help="Adam steps per frame (default: the library's)")
    p.add_argument("--nrc-ema", type=float, default=None, help="moving-average decay of the cache's weights")
    p.add_argument("--nrc-only", action="store_true", help="time-to-relMSE: skip the plain spp ladder")
    # the radiance-cache leg's defaults are the configuration measured fastest
    # to relMSE 0.01 on the 1080p material grid (one frame of 7 spp, paths
    # ending at their first diffuse-ish vertex; 3 spp per frame needs two
    # frames); the library's own defaults (4 spp, ending after it) converge
    # further but reach 0.01 later
    p.add_argument("--nrc-spp", type=int, default=7, help="cached samples per pixel per frame (0: the library's)")
    p.add_argument("--nrc-end-at", type=int, default=1,
                   help="where a cached path ends: 0 after the first diffuse-ish vertex, 1 at it (mt_nrc_config.end_at); "
                        "-1: the library's")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def workload_name(a):
    return f"material_grid_{a.width}x{a.height}_{a.spp}spp"


# --------------------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, smax, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
                power.append(float(f[3]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm), "power_w_max": max(power) if power else None}


# --------------------------------------------------------------------------- CPU baseline
def cpu_baseline(scene, cfg, target_seconds, fast=True):
    """The oracle (restated reference, reference tile queue and threads) on a
    band of rows around the image centre, sized to about target_seconds."""
    from oracle import oracle_py as orc
    import mitrace_gb300 as mt

    threads = os.cpu_count() or 1
    o = orc.OracleScene(mt.PackedScene(scene), cfg, fast=fast)
    H = cfg.height
    rows = 4
    r0 = H // 2 - rows // 2
    t = time.perf_counter()
    _, rays, samples = o.render(orc.RNG_MT19937, threads, r0, r0 + rows)
    dt = time.perf_counter() - t
    rows = max(4, min(H, int(rows * target_seconds / max(dt, 1e-3))))
    r0 = max(0, H // 2 - rows // 2)
    t = time.perf_counter()
    _, rays, samples = o.render(orc.RNG_MT19937, threads, r0, r0 + rows)
    dt = time.perf_counter() - t
    return {
        "value": rays / dt / 1e6,
        "unit": "Mrays/s",
        "cores": threads,
        "kind": "port",
        "sample": f"rows {r0}-{r0 + rows} of {cfg.width}x{H} at {cfg.samples} spp "
                  f"({samples} samples, {rays} rays, {dt:.1f} s, mt19937 per 32x32 tile)",
        "seconds": dt,
        "msamples_s": samples / dt / 1e6,
        "cpu": cpu_model(),
    }


def cpu_model():
    try:
        for ln in open("/proc/cpuinfo"):
            if ln.lower().startswith(("model name", "cpu model")):
                return ln.split(":", 1)[1].strip()
        out = subprocess.run(["lscpu"], capture_output=True, text=True).stdout
        for ln in out.splitlines():
            if "Model name" in ln:
                return ln.split(":", 1)[1].strip()
    except Exception:
        pass
    return os.uname().machine


def run_reference(a):
    import mitrace_gb300.scenes as S

    rank, world, _ = dist_env()
    if rank != 0:
        return
    scene, cfg = S.material_grid(width=a.width, height=a.height, samples=a.spp)
    vals = []
    base = None
    for i in range(a.warmup + a.steps):
        r = cpu_baseline(scene, cfg, a.cpu_seconds / 2 if i < a.warmup else a.cpu_seconds)
        if i >= a.warmup:
            vals.append(r["value"])
            base = r
    v = statistics.median(vals)
    line = {
        "impl": "reference", "metric": "Mrays/s", "value": v, "unit": "Mrays/s", "n_gpus": a.gpus,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": base["seconds"] * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": workload_name(a), "width": a.width, "height": a.height, "spp": a.spp,
                   "note": "reference's CPU path restated (cannot be built here); bounded band per step"},
        "cpu_baseline": {k: base[k] for k in ("value", "unit", "cores", "kind", "sample")} | {"value": v},
        "e2e": {"value": v, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------- microbench
def microbench(a, dev, peak):
    """Incoherent rays (origins uniform in the scene box, directions uniform on
    the sphere, seed 0) against the large scene: fBm terrain of 2 * 1023^2
    triangles plus 50k icospheres of 80 triangles, each set one mesh.  Closest
    hit and any hit through mt_trace_rays_device; device-resident rays and
    hits (> L2), CUDA events on the launching stream."""
    import ctypes as C

    import numpy as np
    import torch

    import mitrace_gb300 as mt
    from mitrace_gb300 import _abi as A

    scene, cfg = mt.large_scene(samples=1)
    lo, hi = mt.scene_bounds(scene)
    n = a.microbench_rays
    rays = mt.incoherent_rays(lo, hi, n, seed=0)
    t0 = time.perf_counter()
    tr = mt.Tracer(scene, cfg)
    create_s = time.perf_counter() - t0
    stream = torch.cuda.current_stream(dev)
    assert stream.cuda_stream != 0
    d_rays = torch.from_numpy(rays).to(dev)
    d_hits = torch.empty((n, 8), dtype=torch.int32, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    out = {"scene": "fBm terrain 2x1023^2 tris + 50k icospheres x 80 tris (merged meshes)",
           "triangles": scene.num_triangles, "rays": n, "create_s": create_s}
    # traversal work of the closest-hit query (untimed counting pass)
    tr.trace_device(d_rays.data_ptr(), n, d_hits.data_ptr(), A.MT_QUERY_CLOSEST_TOTALS, stream.cuda_stream)
    torch.cuda.synchronize()
    h = d_hits.cpu().numpy().view(np.uint32)
    inner, tris = int(h[:, 5].astype(np.uint64).sum()), int(h[:, 7].astype(np.uint64).sum())
    alg_bytes = 64 * inner + 40 * tris + 64 * n
    out["hit_fraction"] = float((h[:, 3] != A.MT_NO_HIT).mean())
    out["per_ray"] = {"inner_pops": inner / n, "tri_tests": tris / n, "node_pops": float(h[:, 6].mean())}
    for name, q in (("closest", A.MT_QUERY_CLOSEST), ("any", A.MT_QUERY_ANY)):
        tr.trace_device(d_rays.data_ptr(), n, d_hits.data_ptr(), q, stream.cuda_stream)  # warm-up
        ms = []
        for i in range(3):
            flush.fill_(i)
            s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s0.record(stream)
            tr.trace_device(d_rays.data_ptr(), n, d_hits.data_ptr(), q, stream.cuda_stream)
            s1.record(stream)
            torch.cuda.synchronize()
            ms.append(s0.elapsed_time(s1))
        t = statistics.median(ms)
        out[f"{name}_mrays_s"] = n / (t / 1e3) / 1e6
        out[f"{name}_ms"] = t
    achieved = alg_bytes / (out["closest_ms"] / 1e3) / 1e9
    out["roofline_closest"] = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                               "frac": achieved / peak, "alg_bytes": alg_bytes}
    tr.close()
    # host BVH build of the scene's meshes: the library's builder (independent
    # subtrees on threads) against the oracle's restatement of the reference's
    # recursive builder; both give the same nodes and indices
    from oracle import oracle_py as orc

    builds = []
    for m in scene.meshes:
        t0 = time.perf_counter()
        n1, i1 = mt.bvh_build(m.positions)
        t1 = time.perf_counter()
        n2, i2 = orc.bvh_build(m.positions)
        t2 = time.perf_counter()
        builds.append({"triangles": int(m.num_triangles), "nodes": int(n1.shape[0]), "library_s": t1 - t0,
                       "reference_restatement_s": t2 - t1,
                       "identical": bool(np.array_equal(n1, n2) and np.array_equal(i1, i2))})
    out["bvh_build"] = builds
    return out


# --------------------------------------------------------------------------- radiance cache kernels
def nrc_microbench(dev, rows=1920 * 1080 * 4):
    """The cache's tensor-core kernels alone: inference over 1920x1080x4
    feature records (one frame's worth of queries at most) and one training
    step of 16,384 rows (forward, backward through the activations, weight
    gradient, Adam).  Algorithmic flop: 2 * 17,600 per row forward; a training
    row adds the backward data pass (2 * 12,480: no input gradient for the
    first layer) and the weight gradient (2 * 17,600).  CUDA events on the
    launching stream, median of 5 after warm-up."""
    import numpy as np
    import torch

    import mitrace_gb300 as mt
    from mitrace_gb300 import _abi as A

    peak = None
    if PEAKS_FILE.exists():
        peak = float(json.loads(PEAKS_FILE.read_text())["bf16_tflops"])
    stream = torch.cuda.current_stream(dev)
    scene, cfg = mt.box_room(width=64, height=64, samples=1)
    out = {}
    with mt.Tracer(scene, cfg) as tr:
        tr.nrc_enable()
        rng = np.random.default_rng(0)
        n = rows
        f = np.zeros((n, 5, 4), np.float32)
        f[:, 0, :] = rng.random((n, 4))
        v = rng.normal(size=(n, 2, 3))
        f[:, 1:3, :3] = v / np.linalg.norm(v, axis=2, keepdims=True)
        f[:, 3:5, :3] = rng.random((n, 2, 3))
        feat = torch.from_numpy(f.reshape(n, 20)).to(dev)
        y = torch.empty((n, 3), device=dev)

        def timed(fn):
            fn()
            ms = []
            for _ in range(5):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                fn()
                e1.record(stream)
                torch.cuda.synchronize()
                ms.append(e0.elapsed_time(e1))
            return statistics.median(ms)

        t = timed(lambda: tr.nrc_infer_device(feat.data_ptr(), n, y.data_ptr(), stream.cuda_stream))
        fl = 2.0 * A.MT_NRC_PARAMS * n
        out["infer"] = {"rows": n, "ms": t, "tflops": fl / t / 1e9, "mqueries_s": n / t / 1e3}
        rows = 16384
        tgt = torch.rand((rows, 3), device=dev)
        t = timed(lambda: tr.nrc_train_step_device(feat.data_ptr(), tgt.data_ptr(), rows, 0, 0, stream.cuda_stream))
        fl = (2.0 * A.MT_NRC_PARAMS * 2 + 2.0 * (3 * 64 * 64 + 64 * 3)) * rows
        out["train_step"] = {"rows": rows, "ms": t, "tflops": fl / t / 1e9}
    if peak:
        for k in ("infer", "train_step"):
            out[k]["frac_of_measured_bf16"] = out[k]["tflops"] / peak
        out["peak_bf16_tflops"] = peak
    return out


def adjoint_bench(dev):
    """mt_render_grad on the inverse-materials scene (7x7 material grid, 512x512,
    64 spp, 512^2 RGB32F albedo texture): one gradient evaluation = the forward
    render plus the path replay and the adjoint, timed with CUDA events."""
    import numpy as np
    import torch

    import mitrace_gb300 as mt

    stream = torch.cuda.current_stream(dev)
    scene, cfg = mt.scenes.adjoint_scene()
    nm, nl = len(scene.materials), len(scene.lights)
    nt = mt.scenes.num_grad_texels(scene)
    target = torch.full((cfg.height, cfg.width, 3), 0.3, device=dev)
    bufs = [torch.zeros(k, device=dev) for k in (cfg.height * cfg.width * 3, 1, nm * 3, nm, nm, max(nl, 1), max(nt, 1))]
    ms = []
    with mt.Tracer(scene, cfg) as tr:
        for i in range(4):
            for b in bufs[2:]:
                b.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            tr.render_grad_device(target.data_ptr(), *[b.data_ptr() for b in bufs], stream.cuda_stream)
            e1.record(stream)
            torch.cuda.synchronize()
            if i:
                ms.append(e0.elapsed_time(e1))
    t = statistics.median(ms)
    samples = cfg.width * cfg.height * cfg.samples
    return {"workload": f"adjoint_material_grid_{cfg.width}x{cfg.height}_{cfg.samples}spp",
            "parameters": nm * 5 + nl + nt, "ms_per_gradient": t, "msamples_per_s": samples / t / 1e3,
            "loss": float(bufs[1].item())}


# --------------------------------------------------------------------------- GPU arm
def run_ours(a):
    import ctypes as C

    import numpy as np
    import torch

    import mitrace_gb300 as mt
    from mitrace_gb300 import _abi as A

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    scene, cfg = mt.material_grid(width=a.width, height=a.height, samples=a.spp)
    tr = mt.Tracer(scene, cfg)
    # an explicit non-default stream: the library enqueues on exactly this
    # stream, so the CUDA events below bracket its kernels
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    sptr = stream.cuda_stream
    assert sptr != 0
    out = torch.empty((a.height, a.width, 3), dtype=torch.float32, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)  # 256 MiB > 129 MB L2

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    # untimed counting pass: traversal work per render (deterministic: fixed seed)
    A.check(A.lib.mt_profile_enable(tr.handle, 0, 1), "profile")
    tr.render_device(out.data_ptr(), sptr)
    prof = A.mt_profile()
    A.check(A.lib.mt_profile_read(tr.handle, C.byref(prof)), "profile_read")
    ext = prof.stage[A.MT_STAGE_EXTEND]
    shd = prof.stage[A.MT_STAGE_SHADOW]
    rays_per_render = int(ext.rays + shd.rays)
    counts = {"extend_rays": int(ext.rays), "shadow_rays": int(shd.rays), "extend_node_pops": int(ext.node_pops),
              "extend_inner_pops": int(ext.inner_pops), "extend_tri_tests": int(ext.tri_tests),
              "shadow_node_pops": int(shd.node_pops), "shadow_inner_pops": int(shd.inner_pops),
              "shadow_tri_tests": int(shd.tri_tests)}
    A.check(A.lib.mt_profile_enable(tr.handle, 0, 0), "profile")
    A.check(A.lib.mt_profile_reset(tr.handle), "profile_reset")

    for _ in range(a.warmup):
        tr.render_device(out.data_ptr(), sptr)
    torch.cuda.synchronize()
    # the warm-up renders must count the same rays as the counting pass
    st = tr.GetStats()
    assert st.rays == rays_per_render, (st.rays, rays_per_render)

    A.check(A.lib.mt_profile_enable(tr.handle, 1, 0), "profile")
    A.check(A.lib.mt_profile_reset(tr.handle), "profile_reset")
    clocks = ClockSampler(local)
    launches0 = tr.kernel_launches()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(a.steps)]
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    for i in range(a.steps):
        flush.fill_(i & 0xFF)  # evict the scene from L2 between steps (not timed)
        ev[i][0].record(stream)
        tr.render_device(out.data_ptr(), sptr)
        ev[i][1].record(stream)
    torch.cuda.synchronize()
    barrier()
    clk = clocks.stop()
    launches = tr.kernel_launches() - launches0
    ms = sum(s.elapsed_time(e) for s, e in ev)
    A.check(A.lib.mt_profile_read(tr.handle, C.byref(prof)), "profile_read")
    st = tr.GetStats()
    assert st.rays == rays_per_render
    ms_t = torch.tensor([ms], dtype=torch.float64, device=dev)
    if world > 1:
        torch.distributed.all_reduce(ms_t, op=torch.distributed.ReduceOp.MAX)
    ms_max = float(ms_t.item())
    total_rays = rays_per_render * a.steps * world
    value = total_rays / (ms_max / 1e3) / 1e6

    # roofline of the extend (closest-hit traversal) kernel
    ext_t = prof.stage[1]
    per_launch_ms = ext_t.milliseconds / max(1, ext_t.launches)
    alg_bytes_render = 64 * counts["extend_inner_pops"] + 40 * counts["extend_tri_tests"] + 48 * counts["extend_rays"]
    launches_per_render = ext_t.launches / a.steps
    bytes_per_launch = alg_bytes_render / launches_per_render
    achieved = bytes_per_launch / (per_launch_ms / 1e3) / 1e9
    peak, peak_src = FALLBACK_HBM_GBS, "fallback"
    if PEAKS_FILE.exists():
        try:
            peak, peak_src = float(json.loads(PEAKS_FILE.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    traffic = None
    if TRAFFIC_FILE.exists():
        # DRAM bytes per extend ray from the ncu summary (a capture of a smaller
        # render of the same scene), times this run's extend rays per launch
        text = TRAFFIC_FILE.read_text()
        w = re.search(r"^traffic_workload: (\S+)$", text, re.M)
        b = re.search(r"^traffic_bytes_per_extend_ray: ([0-9.]+)$", text, re.M)
        if w and b and w.group(1) == workload_name(a):
            traffic = round(float(b.group(1)) * counts["extend_rays"] / launches_per_render)
    stage_ms = {n: round(prof.stage[i].milliseconds / a.steps, 3) for i, n in
                enumerate(["raygen", "extend", "shade", "shadow", "finalize", "resolve"])}

    # e2e through the host API
    e2e_steps = a.e2e_steps if a.e2e_steps is not None else max(1, min(a.steps, 3))
    tr.close()
    del out
    torch.cuda.empty_cache()
    img = np.empty((a.height, a.width, 3), dtype=np.float32)
    t_e2e = []
    for i in range(e2e_steps + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        with mt.Tracer(scene, cfg) as t2:
            t2.StartRender()
            img[...] = t2.WaitForRender()
        torch.cuda.synchronize()
        if i > 0:  # the first one is a warm-up
            t_e2e.append(time.perf_counter() - t0)
    e2e_s = sum(t_e2e)
    e2e_value = rays_per_render * len(t_e2e) / e2e_s / 1e6

    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return
    line = {
        "metric": "Mrays/s",
        "value": value,
        "unit": "Mrays/s",
        "n_gpus": world,
        "steps": a.steps,
        "warmup": a.warmup,
        "ms_per_step": ms_max / a.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": {
            "workload": workload_name(a), "width": a.width, "height": a.height, "spp": a.spp, "bounces": cfg.bounces,
            "triangles": scene.num_triangles, "instances": len(scene.instances), "lights": len(scene.lights),
            "rays_per_step": rays_per_render, "samples_per_step": a.width * a.height * a.spp,
            "l2": "256 MiB buffer written between timed steps (not timed)",
            "parallelism": "replicas" if world > 1 else "single GPU",
        },
        "msamples_per_s": a.width * a.height * a.spp * a.steps * world / (ms_max / 1e3) / 1e6,
        "e2e": {"value": e2e_value, "unit": "Mrays/s", "h2d_bytes_per_step": int(scene.nbytes()),
                "d2h_bytes_per_step": int(img.nbytes), "seconds_per_step": e2e_s / len(t_e2e)},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "kernel": "k_extend", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_source": peak_src,
                     "alg_bytes_per_launch": bytes_per_launch, "launch_ms": per_launch_ms,
                     "launches": int(ext_t.launches)},
        "traversal_counts_per_step": counts,
        "stage_ms_per_step": stage_ms,
        "clocks": clk,
    }
    if not a.no_microbench:
        torch.cuda.empty_cache()
        line["incoherent"] = microbench(a, dev, peak)
        torch.cuda.empty_cache()
        line["nrc_kernels"] = nrc_microbench(dev)
        torch.cuda.empty_cache()
        line["adjoint"] = adjoint_bench(dev)
    if not a.no_cpu_baseline:
        cb = cpu_baseline(scene, cfg, a.cpu_seconds)
        line["cpu_baseline"] = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")}
        line["cpu_baseline"]["cpu"] = cb["cpu"]
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


# --------------------------------------------------------------------------- time to relMSE
def relmse(x, r):
    """Mean over pixels and channels of (x - r)^2 / (r^2 + 1e-2), on the
    tonemapped images the renderer outputs."""
    return float(((x - r) ** 2 / (r * r + 1e-2)).mean())


def run_time_to_relmse(a):
    """Renders the material grid at an spp ladder (seed 0) and a reference at
    --ref-spp (seed 1); reports relMSE per rung, the GPU time to reach the
    target (first rung at or below it, and the 1/spp fit), and the CPU oracle's
    time for the same spp extrapolated from its measured samples/s."""
    import numpy as np
    import torch

    import mitrace_gb300 as mt

    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)

    def render(spp, seed, warm=True):
        scene, cfg = mt.material_grid(width=a.width, height=a.height, samples=spp, seed=0)
        cfg.seed = seed
        out = torch.empty((a.height, a.width, 3), dtype=torch.float32, device=dev)
        with mt.Tracer(scene, cfg) as tr:
            if warm:
                tr.render_device(out.data_ptr(), stream.cuda_stream)  # warm-up
            torch.cuda.synchronize()
            s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s0.record(stream)
            tr.render_device(out.data_ptr(), stream.cuda_stream)
            s1.record(stream)
            torch.cuda.synchronize()
            rays = tr.GetStats().rays
        return out.cpu().numpy(), s0.elapsed_time(s1) / 1e3, rays, scene, cfg

    t0 = time.perf_counter()
    ref, ref_s, ref_rays, scene, cfg = render(a.ref_spp, 1, warm=False)  # seconds-long: no warm-up
    ladder = []
    spp = 1
    while spp <= (0 if a.nrc_only else 1024):
        img, sec, rays, _, _ = render(spp, 0)
        ladder.append({"spp": spp, "seconds": sec, "relmse": relmse(img, ref), "mrays_s": rays / sec / 1e6})
        spp *= 2
    rung = next((r for r in ladder if r["relmse"] <= a.relmse_target), None)
    # the smallest passing spp: every count between the last failing power of
    # two and the first passing one is rendered (with the same seed)
    hit, refine = rung, []
    if rung and rung["spp"] > 1:
        for spp in range(rung["spp"] // 2 + 1, rung["spp"]):
            img, sec, rays, _, _ = render(spp, 0)
            r = {"spp": spp, "seconds": sec, "relmse": relmse(img, ref), "mrays_s": rays / sec / 1e6}
            refine.append(r)
            if r["relmse"] <= a.relmse_target:
                hit = r
                break
    # relMSE ~ c / spp on the rungs above 8 spp
    xs = np.array([r["spp"] for r in ladder if r["spp"] >= 8], dtype=np.float64)
    ys = np.array([r["relmse"] for r in ladder if r["spp"] >= 8], dtype=np.float64)
    c = float(np.exp(np.mean(np.log(ys * xs)))) if xs.size else float("nan")
    spp_fit = c / a.relmse_target
    sec_per_spp = (statistics.median(r["seconds"] / r["spp"] for r in ladder if r["spp"] >= 8) if xs.size
                   else float("nan"))
    line = {
        "metric": "time-to-relMSE 0.01 @1080p", "unit": "s", "higher_is_better": False,
        "config": {"workload": workload_name(a), "ref_spp": a.ref_spp, "ref_seed": 1, "seed": 0,
                   "relmse": "mean over pixels/channels of (x-r)^2/(r^2+1e-2) on the tonemapped output"},
        "gpu_first_rung": rung, "gpu_min_spp": hit, "refine": refine,
        "gpu_fit": {"c": c, "spp": spp_fit, "seconds": spp_fit * sec_per_spp},
        "ladder": ladder, "reference_seconds": ref_s, "reference_rays": ref_rays,
    }
    if not a.no_cpu_baseline and hit:
        # the CPU oracle (reference's CPU path restated, -Ofast, every host core,
        # mt19937 per 32x32 tile) renders the whole image at the same spp
        from oracle import oracle_py as orc

        scene_c, cfg_c = mt.material_grid(width=a.width, height=a.height, samples=hit["spp"], seed=0)
        cfg_c.seed = 0
        threads = os.cpu_count() or 1
        o = orc.OracleScene(mt.PackedScene(scene_c), cfg_c, fast=True)
        t1 = time.perf_counter()
        img_c, rays_c, samples_c = o.render(orc.RNG_MT19937, threads)
        cpu_s = time.perf_counter() - t1
        line["cpu"] = {"spp": hit["spp"], "seconds": cpu_s, "relmse": relmse(img_c, ref), "cores": threads,
                       "cpu": cpu_model(), "mrays_s": rays_c / cpu_s / 1e6,
                       "note": "measured: full image at the GPU's smallest passing spp, same reference"}
        line["speedup_vs_cpu_at_target"] = cpu_s / hit["seconds"]
    if not a.no_nrc:
        line["nrc"] = nrc_time_to_relmse(a, ref, dev, stream)
        if line["nrc"].get("seconds_to_target") and hit:
            line["nrc_vs_plain_time"] = line["nrc"]["seconds_to_target"] / hit["seconds"]
    line["wall_s"] = time.perf_counter() - t0
    print(json.dumps(line), flush=True)


def nrc_time_to_relmse(a, ref, dev, stream):
    """The radiance-cache renderer on the same scene: --nrc-warmup training-only
    frames, then cached frames (--nrc-spp samples per pixel, --nrc-end-at, and
    the mt_nrc_config defaults otherwise: 65,536 training paths and 128 Adam
    steps of 16,384 per frame) folded into a running mean.
    Every frame is timed with CUDA events on the render stream; relMSE of the
    running mean against the plain reference is evaluated between frames,
    outside the timed spans."""
    import torch

    import mitrace_gb300 as mt

    scene, cfg = mt.material_grid(width=a.width, height=a.height, samples=4, seed=0)
    cfg.seed = 0
    refd = torch.from_numpy(ref).to(dev)
    acc = torch.zeros_like(refd)
    out = {"warmup_frames": a.nrc_warmup, "frames": []}
    with mt.Tracer(scene, cfg) as tr:
        kw = {}
        if a.nrc_steps:
            kw["train_steps"] = a.nrc_steps
        if a.nrc_ema is not None:
            kw["ema_decay"] = a.nrc_ema
        if a.nrc_spp and a.nrc_spp > 0:
            kw["spp"] = a.nrc_spp
        if a.nrc_end_at is not None and a.nrc_end_at >= 0:
            kw["end_at"] = a.nrc_end_at
        c = tr.nrc_enable(**kw)
        out["config"] = {"spp_per_frame": c.spp, "train_paths": c.train_paths, "train_batch": c.train_batch,
                         "train_steps": c.train_steps, "lr": c.learning_rate, "rough_min": c.rough_min,
                         "end_at": c.end_at}
        ev = []
        total = 0.0
        for f in range(a.nrc_warmup + a.nrc_frames):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            cached = f >= a.nrc_warmup
            k = f - a.nrc_warmup
            tr.nrc_frame(acc.data_ptr() if cached else 0, max(k, 0), stream.cuda_stream)
            e1.record(stream)
            e1.synchronize()
            ms = e0.elapsed_time(e1)
            total += ms / 1e3
            if not cached:
                out.setdefault("warmup_ms", []).append(ms)
                continue
            r = float(((acc - refd) ** 2 / (refd * refd + 1e-2)).mean().item())
            out["frames"].append({"frame": k, "ms": ms, "cum_s": total, "relmse": r})
            if r <= a.relmse_target and "seconds_to_target" not in out:
                out["seconds_to_target"] = total
                out["frames_to_target"] = k + 1
                if k >= 3:
                    break
    out["best_relmse"] = min(x["relmse"] for x in out["frames"]) if out["frames"] else None
    return out


def main():
    a = parse()
    if a.nrc_kernels_only:
        import torch

        dev = torch.device("cuda", 0)
        torch.cuda.set_stream(torch.cuda.Stream(dev))
        print(json.dumps({"nrc_kernels": nrc_microbench(dev, a.nrc_rows)}), flush=True)
        return
    if a.time_to_relmse:
        run_time_to_relmse(a)
        return
    if a.impl == "reference":
        run_reference(a)
    else:
        run_ours(a)


if __name__ == "__main__":
    main()
