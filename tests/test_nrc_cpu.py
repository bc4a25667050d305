"""Radiance-cache checks that need no GPU: the encoding's spherical harmonics
are orthonormal and the triangle waves periodic (pins the constants of the
reference encoding the GPU tests compare against), the torch reference's
relative-L2 gradient matches its closed form, and the C entry points report
argument errors and defaults."""
import ctypes as C

import numpy as np
import pytest

from mitrace_gb300 import _abi as A
from tests import nrc_reference as ref


def fibonacci_sphere(n):
    i = np.arange(n) + 0.5
    z = 1 - 2 * i / n
    r = np.sqrt(1 - z * z)
    phi = np.pi * (1 + 5 ** 0.5) * i
    return np.stack([r * np.cos(phi), r * np.sin(phi), z], axis=1)


def test_spherical_harmonics_are_orthonormal():
    d = fibonacci_sphere(200_000)
    y = ref.sh16(d).astype(np.float64)
    gram = 4 * np.pi * (y.T @ y) / d.shape[0]
    np.testing.assert_allclose(gram, np.eye(16), atol=2e-3)


def test_harmonics_match_scipy_up_to_sign_convention():
    sp = pytest.importorskip("scipy.special")
    if not hasattr(sp, "sph_harm_y"):
        pytest.skip("scipy without sph_harm_y")
    d = fibonacci_sphere(999)
    theta = np.arccos(np.clip(d[:, 2], -1, 1))
    phi = np.arctan2(d[:, 1], d[:, 0])
    y = ref.sh16(d).astype(np.float64)
    for l in range(4):
        for m in range(-l, l + 1):
            c = sp.sph_harm_y(l, abs(m), theta, phi)
            real = c.real if m == 0 else np.sqrt(2) * (c.real if m > 0 else c.imag)
            # real basis: sin(|m| phi) for m < 0, cos(m phi) for m > 0; signs vary by convention
            np.testing.assert_allclose(np.abs(y[:, l * l + l + m]), np.abs(real), atol=2e-6, err_msg=f"l={l} m={m}")


def test_triangle_octaves():
    f = ref.random_features(512, seed=3).reshape(-1, 5, 4)
    e = ref.encode(f.reshape(-1, 20))
    assert e.shape == (512, 80) and e.dtype == np.float32
    assert np.all(np.abs(e[:, :36]) <= 1.0)
    # octave j has period 2^-j: shifting x by 2^-j leaves it unchanged
    g = f.copy()
    g[:, 0, 0] = np.float32(0.25) + f[:, 0, 0] * np.float32(0.5)  # keep x + 2^-1 inside [0, 1]
    h = g.copy()
    h[:, 0, 0] += np.float32(0.5)
    ok = h[:, 0, 0] <= 1.0
    eg, eh = ref.encode(g.reshape(-1, 20)), ref.encode(h.reshape(-1, 20))
    # (x + 1/2 rounds away up to one low bit of x, which octave 11 scales by 2^13)
    np.testing.assert_allclose(eg[ok, 1:12], eh[ok, 1:12], atol=2e-3)
    np.testing.assert_array_equal(e[:, 77:80], 1.0)
    np.testing.assert_array_equal(e[:, 69:75], f[:, 3:5, :3].reshape(-1, 6))
    np.testing.assert_array_equal(e[:, 75], f[:, 1, 3])
    np.testing.assert_array_equal(e[:, 76], f[:, 2, 3])


def test_relative_l2_gradient_closed_form():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(1)
    y = torch.tensor(rng.normal(size=(64, 3)), dtype=torch.float64, requires_grad=True)
    t = torch.tensor(rng.uniform(0, 2, (64, 3)), dtype=torch.float64)
    ref.relative_l2(y, t).backward()
    yd, td = y.detach().numpy(), t.numpy()
    expect = 2 * (yd - td) / (yd ** 2 + 0.01) / yd.size
    np.testing.assert_allclose(y.grad.numpy(), expect, rtol=1e-12)


def test_torch_reference_shapes_and_param_count():
    torch = pytest.importorskip("torch")
    assert ref.PARAMS == A.MT_NRC_PARAMS == 17600
    p = torch.zeros(ref.PARAMS)
    x = torch.tensor(ref.encode(ref.random_features(8)))
    assert ref.torch_forward(x, p).shape == (8, 3)


def test_config_defaults():
    c = A.mt_nrc_config()
    A.lib.mt_nrc_config_defaults(C.byref(c))
    assert (c.train_paths, c.train_batch, c.train_steps, c.spp) == (65536, 16384, 128, 4)
    assert c.learning_rate == pytest.approx(1e-2) and c.beta1 == pytest.approx(0.9)
    assert c.beta2 == pytest.approx(0.99) and c.rough_min == pytest.approx(0.3)
    assert c.ema_decay == pytest.approx(0.9)


def test_argument_errors():
    c = A.mt_nrc_config()
    A.lib.mt_nrc_config_defaults(C.byref(c))
    assert A.lib.mt_nrc_enable(None, C.byref(c)) == 3
    assert A.lib.mt_nrc_frame(None, None, 0, None) == 3
    assert A.lib.mt_nrc_infer(None, None, 0, None, None) == 3
    assert A.lib.mt_nrc_train_step(None, None, None, 1, None, None, None) == 3
    assert A.lib.mt_nrc_get_params(None, None) == 3
    assert A.lib.mt_nrc_get_stats(None, None) == 3
    assert A.lib.mt_nrc_set_params(None, None) == 3
    assert A.lib.mt_nrc_encode(None, 4, None, None) == 3
    assert A.lib.mt_nrc_encode(None, 0, None, None) == 0  # nothing to do, no device touched
