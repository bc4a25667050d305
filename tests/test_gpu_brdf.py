"""BRDF eval / pdf parity of the CUDA functions with the oracle's restatement of
src/Tracer/BRDF.hpp:9-97 on seeded inputs (relative 1e-5; the only step the
two sides compute differently is Schlick's (1 - cos)^5: the C library's powf
in the oracle, compensated products on the GPU, correctly rounded except near
a rounding tie)."""
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


def sample_queries(n, seed):
    rng = np.random.default_rng(seed)

    def unit(k):
        v = rng.normal(size=(k, 3))
        return v / np.linalg.norm(v, axis=1, keepdims=True)

    q = np.zeros((n, 16), dtype=np.float32)
    N = unit(n)
    V = unit(n)
    V *= np.sign((V * N).sum(1))[:, None]  # viewer above the surface, as GeneratePath meets it
    q[:, 0:3], q[:, 3:6] = V, N
    q[:, 6:9] = rng.uniform(0, 1, (n, 3))
    q[:, 9] = rng.uniform(0, 1, n)
    q[:, 10] = rng.uniform(0, 1, n)
    q[:, 11:16] = rng.random((n, 5))
    return q


def test_brdf_sampling_matches_oracle():
    """GeneratePath's bounce sample (lobe choice, GGX reflection with its cosine
    fallback, cosine sample, mixture pdf) on seeded uniforms: the same lobe for
    all but decisions within an ulp of the specular probability, directions
    within the sinf/cosf rounding, the specular probability to 1e-5, and the
    mixture pdf to 1e-5 relative of the reference functions evaluated at the
    sampled direction.

    The direction goes through sinf/cosf (one sincosf per angle on the GPU),
    whose last-ulp rounding differs between the GPU and the host C library, and
    a near-mirror GGX lobe (alpha
    down to 0.0025) turns a 1e-7 change of direction into percents of pdf, in
    exact arithmetic as in float.  So the pdf is checked where it is defined:
    the oracle's DiffusePdf / SpecularPdf (BRDF.hpp:80-97) and mixture
    (Tracer.cpp:190-194) are evaluated at the GPU's sampled direction."""
    q = sample_queries(200_000, 3)
    g = mt.brdf_sample_batch(q)
    r = orc.brdf_sample(q)
    lg, lr = g[:, 5].view(np.int32), r[:, 5].view(np.int32)
    same = lg == lr
    assert same.mean() > 0.999
    assert set(np.unique(lg)) == {0, 1, 2}  # every branch exercised
    np.testing.assert_allclose(g[same, 0:3], r[same, 0:3], atol=2e-5)
    np.testing.assert_allclose(g[:, 4], r[:, 4], rtol=1e-5)
    # reference pdfs at the GPU's directions: mt_brdf_query = L, V, N, base, roughness, metallic
    bq = np.zeros((q.shape[0], 14), np.float32)
    bq[:, 0:3], bq[:, 3:6], bq[:, 6:9] = g[:, 0:3], q[:, 0:3], q[:, 3:6]
    bq[:, 9:12], bq[:, 12], bq[:, 13] = q[:, 6:9], q[:, 9], q[:, 10]
    e = orc.brdf_batch(bq)
    ps = r[:, 4]
    one = np.float32(1.0)
    mix = ((one - ps) * e[:, 3]).astype(np.float32) + (ps * e[:, 4]).astype(np.float32)
    np.testing.assert_allclose(g[:, 3], mix, rtol=1e-5, atol=1e-12)
    assert np.all(np.einsum("ij,ij->i", g[:, 0:3], q[:, 3:6]) > -1e-6)  # never below the surface
