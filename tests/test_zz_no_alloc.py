"""The allocation-free render entry point (mt_render_rows_noalloc).

It serves callers that must not allocate GPU memory while they render (a fixed
memory budget reserved up front, a frame loop that must not block in the
allocator, an allocator hooked by another library): all its scratch lives in a
static device array.  Called through the C ABI, its rows must equal the rows
mt_render_device produces for the same scene, on two calls in a row (the
second call finds the first call's leftovers in the shared array).  Requests
above the stated path limit are refused.

This file is named so that pytest collects it last."""
import ctypes as C

import numpy as np
import pytest

import mitrace_gb300 as mt
from mitrace_gb300 import _abi as A

pytestmark = pytest.mark.gpu


def test_noalloc_rows_match_render_device():
    torch = pytest.importorskip("torch")
    # 64 x 64 pixels x 16 spp = 65536 paths: the whole image fits one call at the limit
    scene, cfg = mt.box_room(width=64, height=64, samples=16, seed=4)
    with mt.Tracer(scene, cfg) as tr:
        stream = torch.cuda.current_stream().cuda_stream
        ref = torch.zeros((64, 64, 3), dtype=torch.float32, device="cuda")
        tr.render_device(ref.data_ptr(), stream)
        torch.cuda.synchronize()
        ref_np = ref.cpu().numpy()
        assert ref_np.max() > 0.0

        out = torch.full((64, 64, 3), -1.0, dtype=torch.float32, device="cuda")
        # first call: the whole image; second call: a band, over the first call's state
        A.check(A.lib.mt_render_rows_noalloc(tr.handle, 0, 64, C.c_void_p(out.data_ptr()), C.c_void_p(stream)),
                "mt_render_rows_noalloc")
        torch.cuda.synchronize()
        np.testing.assert_array_equal(out.cpu().numpy(), ref_np)

        out2 = torch.full((64, 64, 3), -1.0, dtype=torch.float32, device="cuda")
        A.check(A.lib.mt_render_rows_noalloc(tr.handle, 16, 48, C.c_void_p(out2.data_ptr()), C.c_void_p(stream)),
                "mt_render_rows_noalloc")
        torch.cuda.synchronize()
        got = out2.cpu().numpy()
        np.testing.assert_array_equal(got[16:48], ref_np[16:48])
        # samples of the two calls are counted, as for mt_render_device
        assert tr.GetStats().samples == (64 * 64 + 32 * 64) * 16 + 64 * 64 * 16
        assert (got[:16] == -1.0).all() and (got[48:] == -1.0).all()  # rows outside the band untouched


def test_noalloc_refuses_requests_above_the_limit():
    torch = pytest.importorskip("torch")
    scene, cfg = mt.box_room(width=64, height=64, samples=32, seed=4)
    with mt.Tracer(scene, cfg) as tr:
        out = torch.zeros((64, 64, 3), dtype=torch.float32, device="cuda")
        rc = A.lib.mt_render_rows_noalloc(tr.handle, 0, 64, C.c_void_p(out.data_ptr()), None)
        assert rc == A.MT_ERR_INVALID
        assert "MT_NOALLOC_MAX_PATHS" in A.lib.mt_last_error().decode()
        assert A.lib.mt_render_rows_noalloc(tr.handle, 5, 5, C.c_void_p(out.data_ptr()), None) == A.MT_ERR_INVALID
        # within the limit on the same handle: 32 rows x 64 x 32 spp = 65536
        A.check(A.lib.mt_render_rows_noalloc(tr.handle, 0, 32, C.c_void_p(out.data_ptr()), None), "noalloc")
        torch.cuda.synchronize()
        assert out[:32].max().item() > 0.0
