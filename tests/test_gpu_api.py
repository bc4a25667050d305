"""Robustness of the C ABI on the GPU: allocation failures come back as
MT_ERR_OOM and leave the handle usable, and the statistics a stat thread polls
(Tracer::GetStats, src/Tracer/Tracer.cpp:806-821, polled by StatThread in
src/main.cpp:52-57) stay consistent while another thread renders.

Allocation failures are injected on the host: MT_DEVICE_ALLOC_LIMIT makes any
single device allocation above the given byte count fail as cudaMalloc does
when the device is out of memory, so no test exhausts a shared GPU."""
import ctypes as C
import os
import threading

import numpy as np
import pytest

import mitrace_gb300 as mt
from mitrace_gb300 import _abi as A

pytestmark = pytest.mark.gpu


class alloc_limit:
    def __init__(self, nbytes):
        self.nbytes = nbytes

    def __enter__(self):
        os.environ["MT_DEVICE_ALLOC_LIMIT"] = str(self.nbytes)

    def __exit__(self, *exc):
        os.environ.pop("MT_DEVICE_ALLOC_LIMIT", None)


def test_oom_on_create_is_reported():
    scene, cfg = mt.material_grid(width=32, height=18, samples=1)
    h = C.c_void_p()
    with alloc_limit(64 << 10):  # the sphere's 4096 triangle slots alone are 200 KB
        rc = A.lib.mt_create(mt.PackedScene(scene).ptr(), C.byref(cfg), C.byref(h))
    assert rc == A.MT_ERR_OOM, A.lib.mt_last_error().decode()
    assert not h.value


def test_oom_on_first_render_leaves_a_usable_handle():
    torch = pytest.importorskip("torch")
    scene, cfg = mt.box_room(width=48, height=48, samples=4, seed=3)
    with mt.Tracer(scene, cfg) as tr:  # the box room's scene buffers are a few KB
        out = torch.zeros((48, 48, 3), device="cuda")
        with alloc_limit(1 << 20):  # the wavefront state is far larger
            rc = A.lib.mt_render_device(tr.handle, C.c_void_p(out.data_ptr()), None)
        assert rc == A.MT_ERR_OOM
        assert "out of memory" in A.lib.mt_last_error().decode() or "Allocation" in A.lib.mt_last_error().decode()
        with alloc_limit(1 << 20):
            assert A.lib.mt_start(tr.handle) == A.MT_ERR_OOM
        # without the limit the same handle renders, and matches a fresh handle
        tr.render_device(out.data_ptr(), 0)
        torch.cuda.synchronize()
        with mt.Tracer(scene, cfg) as fresh:
            ref = torch.zeros_like(out)
            fresh.render_device(ref.data_ptr(), 0)
            torch.cuda.synchronize()
        np.testing.assert_array_equal(out.cpu().numpy(), ref.cpu().numpy())
        assert tr.GetStats().rays > 0


def test_stats_polled_while_rendering():
    """A stat thread polls mt_get_stats / mt_is_done while the render thread
    runs device renders and an asynchronous render: every poll succeeds, the
    counters never go backwards within a render, and the final counts are
    exact."""
    torch = pytest.importorskip("torch")
    scene, cfg = mt.box_room(width=96, height=96, samples=16, seed=5)
    with mt.Tracer(scene, cfg) as tr:
        out = torch.zeros((96, 96, 3), device="cuda")
        tr.render_device(out.data_ptr(), 0)
        torch.cuda.synchronize()
        rays_one = tr.GetStats().rays
        assert rays_one > 0
        stop = threading.Event()
        errors, polls = [], [0]

        def poll():
            s = A.mt_stats()
            while not stop.is_set():
                rc = A.lib.mt_get_stats(tr.handle, C.byref(s))
                if rc != A.MT_OK:
                    errors.append(rc)
                if not 0.0 <= s.progress <= 1.0:
                    errors.append(("progress", s.progress))
                A.lib.mt_is_done(tr.handle)
                polls[0] += 1

        t = threading.Thread(target=poll)
        t.start()
        try:
            for _ in range(6):
                tr.render_device(out.data_ptr(), 0)
            torch.cuda.synchronize()
            tr.StartRender()
            img = tr.WaitForRender()
        finally:
            stop.set()
            t.join()
        assert not errors, errors[:5]
        assert polls[0] > 0
        s = tr.GetStats()
        assert s.rays == rays_one  # the last render's rays, as GetStats reports them
        assert s.samples == 96 * 96 * 16
        np.testing.assert_array_equal(img, out.cpu().numpy())


@pytest.mark.parametrize("world", [2, 3])
def test_row_bands_assemble_the_single_gpu_render(world):
    """mt_render_rows_device on one handle per 'rank' (as on separate GPUs):
    the bands of mitrace_gb300.bands.row_bands assemble mt_render_device's
    image bit for bit, and rows outside a band stay untouched."""
    torch = pytest.importorskip("torch")
    from mitrace_gb300.bands import row_bands

    from .helpers import small_grid

    scene, cfg = small_grid(width=96, height=54, samples=4, seed=6)
    with mt.Tracer(scene, cfg) as tr:
        ref = torch.zeros((54, 96, 3), device="cuda")
        tr.render_device(ref.data_ptr(), 0)
        torch.cuda.synchronize()
    img = torch.full((54, 96, 3), -1.0, device="cuda")
    for r0, r1 in row_bands(54, world):
        with mt.Tracer(scene, cfg) as rank_tr:
            band = torch.full((54, 96, 3), -2.0, device="cuda")
            rank_tr.render_rows_device(r0, r1, band.data_ptr(), 0)
            torch.cuda.synchronize()
            assert (band[:r0] == -2.0).all() and (band[r1:] == -2.0).all()
            assert rank_tr.GetStats().samples == (r1 - r0) * 96 * 4
            img[r0:r1] = band[r0:r1]
    np.testing.assert_array_equal(img.cpu().numpy(), ref.cpu().numpy())


def test_set_seed_equals_a_handle_created_with_that_seed():
    torch = pytest.importorskip("torch")
    scene, cfg = mt.box_room(width=40, height=40, samples=4, seed=1)
    with mt.Tracer(scene, cfg) as tr:
        a = torch.zeros((40, 40, 3), device="cuda")
        tr.render_device(a.data_ptr(), 0)
        tr.set_seed(77)
        b = torch.zeros_like(a)
        tr.render_device(b.data_ptr(), 0)
        torch.cuda.synchronize()
    cfg.seed = 77
    with mt.Tracer(scene, cfg) as t2:
        c = torch.zeros_like(a)
        t2.render_device(c.data_ptr(), 0)
        torch.cuda.synchronize()
    assert not torch.equal(a, b)
    np.testing.assert_array_equal(b.cpu().numpy(), c.cpu().numpy())


def test_device_block_cache_reuses_memory_and_releases_it():
    """A handle created after another was destroyed reuses its cached device
    blocks and renders the same image; mt_release_cached_memory hands the
    blocks back (free device memory rises); MT_DEVICE_CACHE_BYTES=0 turns the
    cache off."""
    torch = pytest.importorskip("torch")
    scene, cfg = mt.box_room(width=128, height=128, samples=64, seed=9)
    imgs = []
    for _ in range(2):
        with mt.Tracer(scene, cfg) as tr:
            out = torch.zeros((128, 128, 3), device="cuda")
            tr.render_device(out.data_ptr(), 0)
            torch.cuda.synchronize()
            imgs.append(out.cpu().numpy())
    np.testing.assert_array_equal(imgs[0], imgs[1])
    free_cached = torch.cuda.mem_get_info()[0]
    A.lib.mt_release_cached_memory()
    free_released = torch.cuda.mem_get_info()[0]
    assert free_released > free_cached  # the 1 M-path wavefront went back to the driver
    os.environ["MT_DEVICE_CACHE_BYTES"] = "0"
    try:
        with mt.Tracer(scene, cfg) as tr:
            out = torch.zeros((128, 128, 3), device="cuda")
            tr.render_device(out.data_ptr(), 0)
            torch.cuda.synchronize()
            np.testing.assert_array_equal(out.cpu().numpy(), imgs[0])
    finally:
        os.environ.pop("MT_DEVICE_CACHE_BYTES", None)
