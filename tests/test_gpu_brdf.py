"""BRDF eval / pdf parity of the CUDA functions with the oracle's restatement of
src/Tracer/BRDF.hpp:9-97 on seeded inputs (relative 1e-5; the only inexact step
on either side is powf)."""
import numpy as np
import pytest

import mitrace_gb300 as mt
from oracle import oracle_py as orc

pytestmark = pytest.mark.gpu


def queries(n, seed):
    rng = np.random.default_rng(seed)

    def unit(k):
        v = rng.normal(size=(k, 3))
        return v / np.linalg.norm(v, axis=1, keepdims=True)

    q = np.zeros((n, 14), dtype=np.float32)
    N = unit(n)
    L = unit(n)
    V = unit(n)
    # most pairs in the upper hemisphere, some below (zero branch)
    flip = rng.random(n) < 0.8
    L[flip] *= np.sign((L[flip] * N[flip]).sum(1))[:, None]
    flip = rng.random(n) < 0.8
    V[flip] *= np.sign((V[flip] * N[flip]).sum(1))[:, None]
    q[:, 0:3], q[:, 3:6], q[:, 6:9] = L, V, N
    q[:, 9:12] = rng.uniform(0, 1, (n, 3))
    q[:, 12] = rng.uniform(0, 1, n)
    q[:, 13] = rng.uniform(-0.2, 1.2, n)  # clamps inside BaseReflectivity are exercised
    return q


def test_brdf_batch_matches_oracle():
    q = queries(200_000, 0)
    g = mt.brdf_batch(q)
    r = orc.brdf_batch(q)
    np.testing.assert_allclose(g, r, rtol=1e-5, atol=1e-7)
    assert (r[:, :3] > 0).any(axis=1).mean() > 0.4
