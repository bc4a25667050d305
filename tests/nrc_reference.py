"""Plain NumPy / PyTorch FP32 reference of the radiance cache's network, used
only by the tests: the input encoding (float32, the kernel's operation order),
the MLP (optionally rounding weights and activations to BF16 as the tensor-core
kernels do), the relative L2 loss and one Adam step."""
import numpy as np

IN, WIDTH, PARAMS = 80, 64, 80 * 64 + 3 * 64 * 64 + 64 * 3
SHAPES = [(64, 80), (64, 64), (64, 64), (64, 64), (3, 64)]

_F = np.float32


def sh16(d):
    """Real spherical harmonics of bands 0..3, (n, 3) unit vectors -> (n, 16)."""
    x, y, z = (d[:, k].astype(np.float32) for k in range(3))
    xx, yy, zz = x * x, y * y, z * z
    c = [_F(v) for v in (0.28209479177387814, 0.48860251190291987, 1.0925484305920792, 0.94617469575756,
                         0.31539156525252, 0.54627421529603959, 0.59004358992664352, 2.8906114426405538,
                         0.45704579946446572, 0.3731763325901154, 1.4453057213202769)]
    one, three, five = _F(1), _F(3), _F(5)
    cols = [np.full_like(x, c[0]), -c[1] * y, c[1] * z, -c[1] * x,
            c[2] * x * y, -c[2] * y * z, c[3] * zz - c[4], -c[2] * x * z, c[5] * (xx - yy),
            c[6] * y * (yy - three * xx), c[7] * x * y * z, c[8] * y * (one - five * zz),
            c[9] * z * (five * zz - three), c[8] * x * (one - five * zz), c[10] * z * (xx - yy),
            c[6] * x * (three * yy - xx)]
    return np.stack(cols, axis=1).astype(np.float32)


def encode(feat):
    """(n, 20) feature records -> (n, 80) float32 encoding (mt_nrc_encode)."""
    f = np.asarray(feat, np.float32).reshape(-1, 5, 4)
    n = f.shape[0]
    out = np.zeros((n, IN), np.float32)
    p = np.clip(f[:, 0, :3], _F(0), _F(1))
    for d in range(3):
        s = p[:, d].copy()
        for j in range(12):
            fr = s - np.floor(s)
            out[:, d * 12 + j] = np.abs(_F(4) * fr - _F(2)) - _F(1)
            s = s * _F(2)
    out[:, 36:52] = sh16(f[:, 1, :3])
    out[:, 52:68] = sh16(f[:, 2, :3])
    out[:, 68] = f[:, 0, 3]
    out[:, 69:72] = f[:, 3, :3]
    out[:, 72:75] = f[:, 4, :3]
    out[:, 75] = f[:, 1, 3]
    out[:, 76] = f[:, 2, 3]
    out[:, 77:80] = 1.0
    return out


def split(params):
    """Flat parameter vector -> the five [out][in] weight matrices (views)."""
    ws, off = [], 0
    for o, i in SHAPES:
        ws.append(params[off:off + o * i].reshape(o, i))
        off += o * i
    return ws


def random_features(n, seed=0):
    """Feature records with the value ranges the renderer produces."""
    rng = np.random.default_rng(seed)
    f = np.zeros((n, 5, 4), np.float32)
    f[:, 0, :3] = rng.uniform(0, 1, (n, 3))
    f[:, 0, 3] = rng.uniform(0, 1, n)
    for k in (1, 2):
        v = rng.normal(size=(n, 3))
        f[:, k, :3] = v / np.linalg.norm(v, axis=1, keepdims=True)
    base = rng.uniform(0.04, 1.0, (n, 3))
    m = rng.uniform(0, 1, (n, 1))
    f[:, 3, :3] = base * (1 - m)
    f[:, 4, :3] = 0.04 * (1 - m) + base * m
    f[:, 1, 3] = rng.integers(0, 5, n) / 4.0  # bounce budget left
    f[:, 2, 3] = rng.uniform(0, 1, n)        # cut-off headroom
    return f.reshape(n, 20)


def torch_forward(x, params, bf16=True):
    """x: (n, 80) encoded inputs (torch fp32); params: flat fp32 tensor."""
    import torch

    def rnd(t):
        return t.to(torch.bfloat16).to(torch.float32) if bf16 else t

    ws = []
    off = 0
    for o, i in SHAPES:
        ws.append(rnd(params[off:off + o * i].reshape(o, i)))
        off += o * i
    h = rnd(x)
    for w in ws[:4]:
        h = rnd(torch.relu(h @ w.T))
    return h @ ws[4].T


def relative_l2(y, t):
    """Mean over rows and channels of (y - t)^2 / (y^2 + 0.01), y held constant
    in the denominator."""
    return ((y - t) ** 2 / (y.detach() ** 2 + 0.01)).mean()


def adam_step(w, g, m, v, t, lr=1e-2, b1=0.9, b2=0.99, eps=1e-15):
    """One Adam step in float32, as k_nrc_adam does it."""
    w, g, m, v = (np.asarray(a, np.float32) for a in (w, g, m, v))
    m = _F(b1) * m + (_F(1) - _F(b1)) * g
    v = _F(b2) * v + (_F(1) - _F(b2)) * g * g
    bc1, bc2 = _F(1 - b1 ** t), _F(1 - b2 ** t)
    w = w - _F(lr) * (m / bc1) / (np.sqrt(v / bc2) + _F(eps))
    return w, m, v
