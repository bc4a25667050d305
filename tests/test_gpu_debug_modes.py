"""Debug render modes (Config::DebugMode, src/CLI/Config.hpp:16-40) on the GPU
against the oracle's restatement of ProcessDebugRay and the heatmap
post-processing (src/Tracer/Tracer.cpp:366-488, 650-716), same counter RNG.

* Modes computed from integers, the hit record or the shading frame (test
  counters, path length, albedo, metallic/roughness, normals, colour per
  mesh / triangle / bounding volume, depth): bit-identical images.
* Modes that depend on sinf/cosf/powf results (the sampled first-bounce
  direction, Fresnel, light components, the plain image under a heatmap):
  at least 99% of pixels within 1e-4 absolute + 1e-3 relative.
"""
import ctypes as C

import numpy as np
import pytest

import mitrace_gb300 as mt
from mitrace_gb300 import _abi as A
from oracle import oracle_py as orc

from .helpers import small_grid

pytestmark = pytest.mark.gpu

EXACT = {1: "primary bvh tests", 2: "total bvh tests", 3: "primary triangle tests", 4: "total triangle tests",
         5: "albedo", 6: "metallic roughness", 7: "geometric normal", 8: "shading normal",
         12: "colour per mesh", 13: "colour per triangle", 14: "colour per bounding volume", 15: "bounces",
         16: "depth"}
CLOSE = {9: "direct only", 10: "indirect only", 11: "emission", 17: "first-hit fresnel", 18: "first-hit brdf",
         19: "first-hit pdf", 20: "reflected direction", 21: "pixel standard deviation",
         22: "firefly elimination"}


def render_both(mode, samples=4):
    scene, cfg = small_grid(width=96, height=54, samples=samples, seed=2)
    cfg.debug_mode = mode
    with mt.Tracer(scene, cfg) as tr:
        tr.StartRender()
        img = tr.WaitForRender().copy()
    ref, _, _ = orc.OracleScene(mt.PackedScene(scene), cfg).render(orc.RNG_COUNTER)
    return img, ref


@pytest.mark.parametrize("mode", sorted(EXACT))
def test_exact_debug_modes(mode):
    img, ref = render_both(mode)
    assert np.isfinite(img).all()
    np.testing.assert_array_equal(img, ref, err_msg=EXACT[mode])
    assert img.max() > 0


@pytest.mark.parametrize("mode", sorted(CLOSE))
def test_sampled_debug_modes(mode):
    img, ref = render_both(mode)
    assert np.isfinite(img).all()
    diff = np.abs(img - ref)
    ok = np.all(diff <= 1e-4 + 1e-3 * np.abs(ref), axis=-1)
    assert ok.mean() >= 0.99, f"{CLOSE[mode]}: {ok.mean():.4f} of pixels match; max diff {diff.max():.3g}"


def resolve_gpu(samples, enable, k, mode):
    """mt_resolve_batch: the render's resolve kernel on given samples."""
    s = np.ascontiguousarray(samples, np.float32)
    npix, spp = s.shape[0], s.shape[1]
    out = np.zeros((npix, 3), np.float32)
    A.check(A.lib.mt_resolve_batch(s.ctypes.data, npix, spp, int(enable), float(k), int(mode), out.ctypes.data),
            "mt_resolve_batch")
    return out


def _intensity_samples(intensities):
    i = np.asarray(intensities, np.float32)
    return np.stack([i * np.float32(0.5), i, i * np.float32(1.5)], axis=1).astype(np.float32)


def test_clamp_debug_values_known_answers():
    """Hand-computed answers (CleanupFireflies, Tracer.cpp:490-548): intensities
    {0, 0, 0, 3} have mean 0.75, population sigma sqrt(1.6875) = 1.2990381, and
    with k = 1 the sample at 3 is the one dropped; intensities 8 x 1, 2 x 21 have
    mean 5, sigma 8, and k = 1 drops both 21s."""
    px = np.stack([_intensity_samples([0, 0, 0, 3]), _intensity_samples([2, 2, 2, 2])])
    sd = resolve_gpu(px, True, 1.0, 21)
    np.testing.assert_allclose(sd[0], [1.2990381] * 3, rtol=1e-6)
    np.testing.assert_array_equal(sd[1], np.zeros(3, np.float32))
    dropped = resolve_gpu(px, True, 1.0, 22)
    np.testing.assert_array_equal(dropped, np.float32([[1, 1, 1], [0, 0, 0]]))
    np.testing.assert_array_equal(resolve_gpu(px, True, 2.0, 22)[0], np.zeros(3, np.float32))
    ten = _intensity_samples([1] * 8 + [21, 21])[None]
    np.testing.assert_array_equal(resolve_gpu(ten, True, 1.0, 22), np.float32([[2, 2, 2]]))
    # without the clamp both modes average the plain samples
    for mode in (21, 22):
        np.testing.assert_allclose(resolve_gpu(px, False, 1.0, mode), px.astype(np.float64).mean(axis=1), rtol=1e-6)


@pytest.mark.parametrize("mode", [0, 21, 22])
@pytest.mark.parametrize("enable,k", [(True, 4.0), (True, 1.5), (False, 6.0)])
def test_resolve_matches_oracle_on_random_samples(mode, enable, k):
    """Random heavy-tailed samples (ragged spp): the GPU resolve and the oracle's
    CleanupFireflies restatement agree bit for bit."""
    rng = np.random.default_rng(11 + mode)
    for spp in (1, 7, 64):
        s = (rng.pareto(1.5, size=(257, spp, 3)) * 0.2).astype(np.float32)
        got = resolve_gpu(s, enable, k, mode)
        ref = np.stack([orc.resolve_pixel(s[i], enable, k, debug_mode=mode) for i in range(s.shape[0])])
        np.testing.assert_array_equal(got, ref)


def test_heatmap_spans_the_ramp():
    img, _ = render_both(4)  # total triangle tests
    # the hottest pixel is red (1, 0, 0); misses are blue (0, 0, 1)
    assert np.any(np.all(img == np.array([1, 0, 0], np.float32), axis=-1))
    assert np.any(np.all(img == np.array([0, 0, 1], np.float32), axis=-1))


def test_debug_modes_rejected_where_unsupported():
    scene, cfg = small_grid(width=32, height=18, samples=2, seed=2)
    cfg.debug_mode = 5
    with mt.Tracer(scene, cfg) as tr:
        c = A.mt_nrc_config()
        A.lib.mt_nrc_config_defaults(C.byref(c))
        assert A.lib.mt_nrc_enable(tr.handle, C.byref(c)) == A.MT_ERR_INVALID
        assert A.lib.mt_render_rows_noalloc(tr.handle, 0, 1, None, None) == A.MT_ERR_INVALID
