"""The neural radiance cache on the GPU, through the C ABI.

1. mt_nrc_encode equals the float32 reference encoding.
2. mt_nrc_infer (fused BF16 tensor-core MLP) equals a plain PyTorch FP32
   forward of the same weights with BF16 rounding of weights and activations,
   to 1e-2 relative in norm; full and ragged row counts.
3. mt_nrc_train_step's gradient equals PyTorch autograd of the relative L2
   loss through that forward to 3e-2 relative per layer, its loss to 1e-3, and
   its Adam update equals the float32 Adam formula applied to that gradient.
4. Training on a smooth target lowers the loss tenfold.
5. With no diffuse-ish vertex (rough_min > 1) a cached frame is bit-identical
   to mt_render_device at the same samples: the cache hooks leave the plain
   estimator untouched.
6. Cached frames on the box room converge near the plain render, for both
   end points of a cached path (mt_nrc_config.end_at).
7. mt_nrc_config.target_cap bounds the training targets: with a cap near zero
   the trained cache returns about nothing.
"""
import numpy as np
import pytest

import mitrace_gb300 as mt
from mitrace_gb300 import _abi as A
from tests import nrc_reference as ref

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()


def small_room(**kw):
    return mt.box_room(width=48, height=48, samples=4, seed=2, **kw)


@pytest.fixture(scope="module")
def tracer():
    scene, cfg = small_room()
    tr = mt.Tracer(scene, cfg)
    tr.nrc_enable(train_paths=4096, train_batch=4096, spp=4)
    yield tr
    tr.close()


def test_encoding_matches_reference():
    f = ref.random_features(3001, seed=4)
    out = torch.zeros((3001, 80), device="cuda")
    fd = dev(f)
    mt.nrc_encode_device(fd.data_ptr(), 3001, out.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    np.testing.assert_allclose(out.cpu().numpy(), ref.encode(f), atol=2e-6, rtol=1e-6)


@pytest.mark.parametrize("n", [4096, 1000, 17])
def test_inference_matches_torch_fp32(tracer, n):
    p = tracer.nrc_get_params()
    f = ref.random_features(n, seed=n)
    out = torch.zeros((n, 3), device="cuda")
    fd = dev(f)
    tracer.nrc_infer_device(fd.data_ptr(), n, out.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    y = out.cpu().numpy().astype(np.float64)
    x = torch.tensor(ref.encode(f))
    r = ref.torch_forward(x, torch.tensor(p)).numpy().astype(np.float64)
    assert np.all(np.isfinite(y))
    assert np.linalg.norm(y - r) <= 1e-2 * np.linalg.norm(r)
    # and it is not the unrounded network either by accident: both close
    r32 = ref.torch_forward(x, torch.tensor(p), bf16=False).numpy()
    assert np.linalg.norm(y - r32) <= 5e-2 * np.linalg.norm(r32)


def test_train_step_gradient_loss_and_adam(tracer):
    n = 3000
    rng = np.random.default_rng(5)
    p0 = (rng.normal(size=A.MT_NRC_PARAMS) * 0.15).astype(np.float32)
    tracer.nrc_set_params(p0)
    f = ref.random_features(n, seed=6)
    t = rng.uniform(0.0, 2.0, (n, 3)).astype(np.float32)
    loss = torch.zeros(1, device="cuda")
    grad = torch.zeros(A.MT_NRC_PARAMS, device="cuda")
    fd, td = dev(f), dev(t)
    tracer.nrc_train_step_device(fd.data_ptr(), td.data_ptr(), n, loss.data_ptr(), grad.data_ptr(),
                                 torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    g = grad.cpu().numpy()
    p1 = tracer.nrc_get_params()
    # torch autograd through the BF16-rounded forward
    pt = torch.tensor(p0, requires_grad=True)
    y = ref.torch_forward(torch.tensor(ref.encode(f)), pt)
    lt = ref.relative_l2(y, torch.tensor(t))
    lt.backward()
    gr = pt.grad.numpy()
    assert abs(float(loss.item()) - float(lt.item())) <= 1e-3 * float(lt.item())
    off = 0
    for l, (o, i) in enumerate(ref.SHAPES):
        a, b = g[off:off + o * i], gr[off:off + o * i]
        assert np.linalg.norm(a - b) <= 3e-2 * np.linalg.norm(b), f"layer {l}"
        off += o * i
    w, _, _ = ref.adam_step(p0, g, np.zeros_like(g), np.zeros_like(g), 1)
    np.testing.assert_allclose(p1, w, atol=1e-6, rtol=1e-6)


def test_training_fits_a_smooth_target():
    scene, cfg = small_room()
    with mt.Tracer(scene, cfg) as tr:
        tr.nrc_enable(train_batch=4096)
        n = 8192
        f = ref.random_features(n, seed=9)
        ff = f.reshape(n, 5, 4)
        t = np.stack([0.5 + 0.4 * np.sin(4 * ff[:, 0, 0]), 0.3 + 0.2 * ff[:, 2, 1], ff[:, 3, 0] + 0.1], 1)
        fd, td = dev(f), dev(t.astype(np.float32))
        loss = torch.zeros(1, device="cuda")
        first = None
        for k in range(300):
            tr.nrc_train_step_device(fd.data_ptr(), td.data_ptr(), n, loss.data_ptr(), 0,
                                     torch.cuda.current_stream().cuda_stream)
            if k == 0:
                torch.cuda.synchronize()
                first = float(loss.item())
        torch.cuda.synchronize()
        last = float(loss.item())
    assert np.isfinite(last) and last < first / 10, (first, last)


@pytest.mark.parametrize("end_at", [A.MT_NRC_END_AFTER_DIFFUSE, A.MT_NRC_END_AT_DIFFUSE])
def test_cache_hooks_leave_plain_paths_unchanged(end_at):
    scene, cfg = small_room()
    img = torch.zeros((cfg.height, cfg.width, 3), device="cuda")
    acc = torch.zeros_like(img)
    st = torch.cuda.current_stream().cuda_stream
    with mt.Tracer(scene, cfg) as tr:
        tr.render_device(img.data_ptr(), st)
        tr.nrc_enable(train_paths=2048, train_batch=1024, spp=cfg.samples, rough_min=2.0, end_at=end_at)
        tr.nrc_frame(acc.data_ptr(), 0, st)
        torch.cuda.synchronize()
    np.testing.assert_array_equal(acc.cpu().numpy(), img.cpu().numpy())


def test_cached_frames_are_reproducible():
    """A frame trains on the cache's own stream beside its render, whose cache
    queries wait for the training; the training vertices are placed in path
    order and the gradient sums have a fixed order.  Two handles with the same
    scene and cache configuration render the same two frames bit for bit."""
    scene, cfg = small_room()
    st = torch.cuda.current_stream().cuda_stream
    accs = []
    for _ in range(2):
        acc = torch.zeros((cfg.height, cfg.width, 3), device="cuda")
        with mt.Tracer(scene, cfg) as tr:
            tr.nrc_enable(train_paths=4096, train_batch=1024, train_steps=16, spp=cfg.samples)
            for f in range(2):
                tr.nrc_frame(acc.data_ptr(), f, st)
            torch.cuda.synchronize()
        accs.append(acc.cpu().numpy())
    assert np.abs(accs[0]).max() > 0
    np.testing.assert_array_equal(accs[0], accs[1])


@pytest.mark.parametrize("end_at", [A.MT_NRC_END_AFTER_DIFFUSE, A.MT_NRC_END_AT_DIFFUSE])
def test_cached_frames_converge_near_plain_render(end_at):
    """Box room at +15 EV, where the per-sample ACES curve is linear (so the
    cache's expectation and the plain estimator's agree; at normal exposure the
    per-sample tonemap of a random suffix and of its mean differ by the Jensen
    gap of the curve).  The cached frames' mean brightness matches the plain
    render within 3% and their relative error is well below that of a render
    whose cache returns zero (paths cut at the query vertex).  Both end points:
    the vertex after the first diffuse-ish one (cache = its outgoing radiance)
    and the first diffuse-ish vertex itself (every vertex of the room; cache =
    the indirect light it reflects, its NEE traced)."""
    def room(spp):
        scene, cfg = mt.box_room(width=64, height=64, samples=spp, seed=2)
        cfg.ev_exposure = 15.0
        return scene, cfg

    st = torch.cuda.current_stream().cuda_stream
    scene, cfg = room(1024)
    plain = torch.zeros((cfg.height, cfg.width, 3), device="cuda")
    with mt.Tracer(scene, cfg) as tr:
        tr.render_device(plain.data_ptr(), st)
        torch.cuda.synchronize()
    p = plain.cpu().numpy().astype(np.float64)
    eps = (0.1 * p.mean()) ** 2

    def cached(zero):
        scene, cfg = room(4)
        acc = torch.zeros_like(plain)
        with mt.Tracer(scene, cfg) as tr:
            tr.nrc_enable(train_paths=16384, train_batch=4096, spp=4, train_steps=8, end_at=end_at)
            if zero:
                tr.nrc_set_params(np.zeros(A.MT_NRC_PARAMS, np.float32))
            for _ in range(0 if zero else 32):  # training only
                tr.nrc_frame(0, 0, st)
            for k in range(32):
                tr.nrc_frame(acc.data_ptr(), k, st)
            torch.cuda.synchronize()
            stats = tr.nrc_get_stats()
        return acc.cpu().numpy().astype(np.float64), stats

    a, stats = cached(False)
    z, _ = cached(True)
    assert np.all(np.isfinite(a))
    assert stats["frames"] == 64 and stats["queries"] > 0 and stats["train_samples"] > 0
    assert np.isfinite(stats["train_loss"])
    rel = float(((a - p) ** 2 / (p * p + eps)).mean())
    rel0 = float(((z - p) ** 2 / (p * p + eps)).mean())
    assert abs(a.mean() / p.mean() - 1) < 0.03, (a.mean(), p.mean())
    assert rel < 0.5 * rel0, (rel, rel0)


def test_target_cap_bounds_training_targets():
    """Two caches trained on the same box-room paths, one with target_cap near
    zero (every target is then about 0) and one without a cap: the capped
    cache's outputs on the same inputs are a small fraction of the uncapped
    one's, so the cap reaches the target computation."""
    scene, cfg = small_room()
    st = torch.cuda.current_stream().cuda_stream
    f = ref.random_features(4096, seed=11)
    fd = dev(f)

    def trained_outputs(cap):
        with mt.Tracer(scene, cfg) as tr:
            tr.nrc_enable(train_paths=4096, train_batch=2048, spp=4, train_steps=32, target_cap=cap)
            for _ in range(8):  # training only
                tr.nrc_frame(0, 0, st)
            out = torch.zeros((4096, 3), device="cuda")
            tr.nrc_infer_device(fd.data_ptr(), 4096, out.data_ptr(), st)
            torch.cuda.synchronize()
            return out.cpu().numpy().astype(np.float64)

    capped = trained_outputs(1e-7)
    free = trained_outputs(0.0)
    assert np.all(np.isfinite(capped)) and np.all(np.isfinite(free))
    assert np.abs(free).mean() > 1e-2, np.abs(free).mean()
    assert np.abs(capped).mean() < 0.1 * np.abs(free).mean(), (np.abs(capped).mean(), np.abs(free).mean())


def test_bounded_tensor_core_wait_reports_timeout_and_handle_recovers():
    """MT_NRC_WAIT_LIMIT=0 makes every in-loop mbarrier wait of the inference
    kernel give up at once, as if the tensor cores never answered: the kernel
    skips its remaining tiles, waits (with the full bound) for its last MMA,
    frees its TMEM and returns; mt_nrc_get_stats reports MT_ERR_TIMEOUT once,
    and the same handle then infers and renders normally."""
    import ctypes as C
    import os

    scene, cfg = mt.box_room(width=32, height=32, samples=2, seed=3)
    with mt.Tracer(scene, cfg) as tr:
        tr.nrc_enable(train_paths=2048, train_batch=2048, spp=2)
        n = 1000
        fd = dev(ref.random_features(n, seed=9))
        out = torch.zeros((n, 3), device="cuda")
        stream = torch.cuda.current_stream().cuda_stream
        tr.nrc_infer_device(fd.data_ptr(), n, out.data_ptr(), stream)
        torch.cuda.synchronize()
        good = out.cpu().numpy().copy()
        os.environ["MT_NRC_WAIT_LIMIT"] = "0"
        try:
            out.zero_()
            tr.nrc_infer_device(fd.data_ptr(), n, out.data_ptr(), stream)
            torch.cuda.synchronize()
        finally:
            os.environ.pop("MT_NRC_WAIT_LIMIT", None)
        st = A.mt_nrc_stats()
        assert A.lib.mt_nrc_get_stats(tr.handle, C.byref(st)) == A.MT_ERR_TIMEOUT
        assert "bounded wait" in A.lib.mt_last_error().decode()
        assert np.all(out.cpu().numpy() == 0.0)  # no tile was written
        # reported once; the handle works again
        assert A.lib.mt_nrc_get_stats(tr.handle, C.byref(st)) == A.MT_OK
        tr.nrc_infer_device(fd.data_ptr(), n, out.data_ptr(), stream)
        img = torch.zeros((32, 32, 3), device="cuda")
        tr.render_device(img.data_ptr(), stream)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(out.cpu().numpy(), good)
        assert img.max().item() > 0
        assert A.lib.mt_nrc_get_stats(tr.handle, C.byref(st)) == A.MT_OK


def test_cache_spp_above_the_handle_samples_regrows_the_wavefront():
    """mt_nrc_enable with more samples per frame than the handle was created
    for resizes the wavefront to one batch per frame; the cached frame (no
    diffuse-ish vertex) still equals the plain render at that spp, and the
    handle's own renders are unchanged."""
    scene, cfg = mt.box_room(width=48, height=48, samples=2, seed=2)
    st = torch.cuda.current_stream().cuda_stream
    before = torch.zeros((48, 48, 3), device="cuda")
    after = torch.zeros_like(before)
    acc = torch.zeros_like(before)
    with mt.Tracer(scene, cfg) as tr:
        tr.render_device(before.data_ptr(), st)
        tr.nrc_enable(train_paths=2048, train_batch=1024, spp=6, rough_min=2.0)
        tr.nrc_frame(acc.data_ptr(), 0, st)
        tr.render_device(after.data_ptr(), st)
        torch.cuda.synchronize()
    cfg6 = mt.box_room(width=48, height=48, samples=6, seed=2)[1]
    ref6 = torch.zeros_like(before)
    with mt.Tracer(scene, cfg6) as tr6:
        tr6.render_device(ref6.data_ptr(), st)
        torch.cuda.synchronize()
    np.testing.assert_array_equal(acc.cpu().numpy(), ref6.cpu().numpy())
    np.testing.assert_array_equal(after.cpu().numpy(), before.cpu().numpy())


def test_misaligned_feature_records_are_rejected():
    import ctypes as C

    scene, cfg = small_room()
    with mt.Tracer(scene, cfg) as tr:
        tr.nrc_enable(train_paths=2048, train_batch=1024, spp=2)
        f = torch.zeros(4 * 20 + 1, device="cuda")
        out = torch.zeros(4 * 3, device="cuda")
        rc = A.lib.mt_nrc_infer(tr.handle, C.c_void_p(f.data_ptr() + 4), 4, C.c_void_p(out.data_ptr()), None)
        assert rc == A.MT_ERR_INVALID and "aligned" in A.lib.mt_last_error().decode()
