"""Known-answer tests that pin the CPU oracle (no GPU).

The reference ships no unit tests or golden vectors, so the oracle is pinned
against the mathematics it restates: published Philox4x32-10 vectors,
Moller-Trumbore hits with known answers, BRDF pdf normalisation, the ACES fit,
the firefly clamp on hand-made samples, and the BVH rules of
src/Scene/BVH.cpp.  The product's host BVH builder is checked against the
oracle's builder here too (it is host code and needs no GPU)."""
import math

import numpy as np
import pytest

import mitrace_gb300 as mt
from mitrace_gb300 import _abi as A
from oracle import oracle_py as orc


# --------------------------------------------------------------------------- Philox
@pytest.mark.parametrize(
    "ctr,key,expect",
    [
        ([0, 0, 0, 0], [0, 0], [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]),
        ([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2, [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]),
        ([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0],
         [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]),
    ],
)
def test_philox_published_vectors(ctr, key, expect):
    assert list(orc.philox(ctr, key)) == expect


# --------------------------------------------------------------------------- ray/triangle
def one_triangle_scene(v0, v1, v2):
    pos = np.array([[v0, v1, v2]], dtype=np.float32)
    nrm = np.array([[[0, 0, 1]] * 3], dtype=np.float32)
    s = mt.SceneData([mt.MeshData(pos, nrm)], [mt.InstanceData(0, 0)], [mt.MaterialData()])
    cfg = mt.make_config(width=4, height=4, samples=1)
    return orc.OracleScene(mt.PackedScene(s), cfg)


def ray(o, d, tmax=3.0e38):
    return [*o, tmax, *d, 0.0]


def test_moller_trumbore_known_answers():
    o = one_triangle_scene((0, 0, 0), (1, 0, 0), (0, 1, 0))
    rays = np.array(
        [
            ray((0.25, 0.25, 1), (0, 0, -1)),  # interior
            ray((0.5, 0.0, 1), (0, 0, -1)),  # on edge v0-v1 (inclusive)
            ray((0.0, 0.0, 1), (0, 0, -1)),  # on vertex v0
            ray((0.6, 0.6, 1), (0, 0, -1)),  # outside: u + v > 1
            ray((0.2, 0.2, 0), (1, 0, 0)),  # parallel: |det| <= eps
            ray((0.25, 0.25, 1), (0, 0, 1)),  # triangle behind the origin: t < 0
            ray((0.25, 0.5, -2), (0, 0, 1)),  # det < 0 branch (from below)
        ],
        dtype=np.float32,
    )
    h = o.trace(rays)
    f = h.view(np.float32)
    hit = h[:, 3] != A.MT_NO_HIT
    # Ray 2 is culled by the instance box: its origin lies on the box's x = 0
    # plane and d.x = 0, so (lo.x - o.x) * (1 / d.x) = 0 * inf = NaN, and
    # max(x, y) = (x < y) ? y : x keeps a NaN in its first argument
    # (IntersectRayAABB, Intersect.cpp:9-18).  Ray 1 has the NaN in the y slot,
    # where the same max drops it, so it reaches the triangle.
    assert hit.tolist() == [True, True, False, False, False, False, True]
    np.testing.assert_array_equal(f[0, :3], np.float32([1.0, 0.25, 0.25]))
    np.testing.assert_array_equal(f[1, :3], np.float32([1.0, 0.5, 0.0]))
    np.testing.assert_array_equal(f[6, :3], np.float32([2.0, 0.25, 0.5]))


def test_vertex_hit_is_inclusive():
    # a second, distant triangle widens the box so the vertex ray is not culled
    pos = np.array([[(0, 0, 0), (1, 0, 0), (0, 1, 0)], [(-3, -3, -5), (-2, -3, -5), (-3, -2, -5)]],
                   dtype=np.float32)
    nrm = np.zeros_like(pos)
    nrm[..., 2] = 1
    s = mt.SceneData([mt.MeshData(pos, nrm)], [mt.InstanceData(0, 0)], [mt.MaterialData()])
    o = orc.OracleScene(mt.PackedScene(s), mt.make_config(width=4, height=4, samples=1))
    h = o.trace(np.array([ray((0, 0, 1), (0, 0, -1))], dtype=np.float32))
    assert h[0, 3] == 0 and h[0, 4] == 0
    np.testing.assert_array_equal(h.view(np.float32)[0, :3], np.float32([1.0, 0.0, 0.0]))


def test_any_hit_uses_closest_distance_compare():
    o = one_triangle_scene((0, 0, 0), (1, 0, 0), (0, 1, 0))
    rays = np.array([ray((0.25, 0.25, 1), (0, 0, -1), 1.5), ray((0.25, 0.25, 1), (0, 0, -1), 0.5),
                     ray((0.25, 0.25, 1), (0, 0, -1), 1.0)], dtype=np.float32)
    h = o.trace(rays, query=A.MT_QUERY_ANY)
    # occluded iff the closest hit lies at distance <= tmax (Tracer.cpp:322)
    assert h[:, 3].tolist() == [1, 0, 1]


# --------------------------------------------------------------------------- BRDF
def _hemisphere_grid(n_theta=300, n_phi=600):
    th = (np.arange(n_theta) + 0.5) / n_theta * (np.pi / 2)
    ph = (np.arange(n_phi) + 0.5) / n_phi * (2 * np.pi)
    T, P = np.meshgrid(th, ph, indexing="ij")
    L = np.stack([np.sin(T) * np.cos(P), np.sin(T) * np.sin(P), np.cos(T)], -1).reshape(-1, 3)
    dw = (np.sin(T) * (np.pi / 2 / n_theta) * (2 * np.pi / n_phi)).reshape(-1)
    return L, dw


def _queries(L, V, N, base, rough, metal):
    n = L.shape[0]
    q = np.zeros((n, 14), dtype=np.float32)
    q[:, 0:3] = L
    q[:, 3:6] = V
    q[:, 6:9] = N
    q[:, 9:12] = base
    q[:, 12] = rough
    q[:, 13] = metal
    return q


@pytest.mark.parametrize("rough", [0.3, 0.6, 1.0])
def test_pdfs_integrate_to_one(rough):
    L, dw = _hemisphere_grid()
    V = np.array([0.0, 0.0, 1.0], dtype=np.float32)
    N = np.array([0.0, 0.0, 1.0], dtype=np.float32)
    r = orc.brdf_batch(_queries(L, V, N, (0.5, 0.5, 0.5), rough, 0.0))
    diffuse = float((r[:, 3].astype(np.float64) * dw).sum())
    spec = float((r[:, 4].astype(np.float64) * dw).sum())
    assert abs(diffuse - 1.0) < 2e-3
    # GGX half-vector pdf mapped to L.  At normal incidence L leaves the
    # hemisphere when the half-vector tilts past 45 degrees, i.e. tan^2 > 1,
    # which under the GGX distribution (alpha = roughness^2) has probability
    # alpha^2 / (1 + alpha^2); the integral over the hemisphere is the rest.
    alpha = max(rough, 0.05) ** 2
    assert abs(spec - 1.0 / (1.0 + alpha * alpha)) < 5e-3


def test_brdf_formula_matches_float64_restatement():
    rng = np.random.default_rng(1)
    n = 2000
    N = np.tile([0.0, 0.0, 1.0], (n, 1))
    L = rng.normal(size=(n, 3))
    L[:, 2] = np.abs(L[:, 2])
    L /= np.linalg.norm(L, axis=1, keepdims=True)
    V = rng.normal(size=(n, 3))
    V[:, 2] = np.abs(V[:, 2])
    V /= np.linalg.norm(V, axis=1, keepdims=True)
    base = rng.uniform(0, 1, (n, 3))
    rough = rng.uniform(0.05, 1, n)
    metal = rng.uniform(0, 1, n)
    q = _queries(L, V, N, base, 0.0, 0.0)
    q[:, 12] = rough
    q[:, 13] = metal
    r = orc.brdf_batch(q).astype(np.float64)
    # float64 restatement of BRDF.hpp:52-77
    Lq, Vq, Nq = (q[:, 0:3].astype(np.float64), q[:, 3:6].astype(np.float64), q[:, 6:9].astype(np.float64))
    B = q[:, 9:12].astype(np.float64)
    R = np.maximum(q[:, 12].astype(np.float64), 0.05)
    M = q[:, 13].astype(np.float64)
    nl = np.maximum((Nq * Lq).sum(1), 0)
    nv = np.maximum((Nq * Vq).sum(1), 0)
    H = Vq + Lq
    H /= np.linalg.norm(H, axis=1, keepdims=True)
    nh = np.clip((Nq * H).sum(1), 0, 1)
    hv = np.clip((H * Vq).sum(1), 0, 1)
    f0 = 0.04 * (1 - np.clip(M, 0, 1))[:, None] + B * np.clip(M, 0, 1)[:, None]
    F = f0 + (1 - f0) * ((1 - hv) ** 5)[:, None]
    a2 = (R * R) ** 2
    D = a2 / (np.pi * (nh * nh * (a2 - 1) + 1) ** 2)
    k = (R + 1) ** 2 / 8
    G = (nv / (nv * (1 - k) + k)) * (nl / (nl * (1 - k) + k))
    kd = (1 - F) * (1 - M)[:, None]
    f = kd * B / np.pi + (D * G)[:, None] * F / np.maximum(4 * nv * nl, 1e-3)[:, None]
    ok = (nl > 1e-3) & (nv > 1e-3)
    np.testing.assert_allclose(r[ok, :3], f[ok], rtol=2e-4, atol=1e-6)
    np.testing.assert_allclose(r[:, 3], nl / np.pi, rtol=1e-5, atol=1e-7)


# --------------------------------------------------------------------------- ACES, firefly
@pytest.mark.parametrize("x", [0.0, 0.01, 0.18, 1.0, 4.0, 100.0])
def test_aces_fit(x):
    c = np.float64(x) * 0.5
    expect = (c * (2.51 * c + 0.03)) / (c * (2.43 * c + 0.59) + 0.14)
    got = orc.aces([x, x, x], 0.5)
    np.testing.assert_allclose(got, [expect] * 3, rtol=1e-6, atol=1e-7)


def test_firefly_clamp_rejects_outlier_and_keeps_count():
    s = np.full((100, 3), 0.5, dtype=np.float32)
    s[17] = 100.0
    np.testing.assert_array_equal(orc.resolve_pixel(s, True, 4.0), np.float32([0.5] * 3))
    mean = (np.float32(0.5) * 99 + np.float32(100.0)) / 100
    np.testing.assert_allclose(orc.resolve_pixel(s, True, 100.0), [mean] * 3, rtol=1e-6)
    np.testing.assert_allclose(orc.resolve_pixel(s, False, 4.0), [mean] * 3, rtol=1e-6)


def _intensity_samples(intensities):
    """Samples whose channels differ but whose (r+g+b)/3 is the given value."""
    i = np.asarray(intensities, np.float32)
    return np.stack([i * np.float32(0.5), i, i * np.float32(1.5)], axis=1).astype(np.float32)


def test_debug_pixel_standard_deviation_known_answer():
    # intensities {0, 0, 0, 3}: mean 0.75, population variance
    # (3 * 0.75^2 + 2.25^2) / 4 = 1.6875, sigma = sqrt(1.6875) = 1.2990381
    s = _intensity_samples([0, 0, 0, 3])
    got = orc.resolve_pixel(s, True, 1.0, debug_mode=21)
    np.testing.assert_allclose(got, [1.2990381] * 3, rtol=1e-6)
    # sigma is taken before any sample is dropped, whatever k is
    np.testing.assert_allclose(orc.resolve_pixel(s, True, 0.0, debug_mode=21), [1.2990381] * 3, rtol=1e-6)
    # constant samples: sigma 0
    np.testing.assert_array_equal(orc.resolve_pixel(_intensity_samples([2, 2, 2]), True, 4.0, debug_mode=21),
                                  np.zeros(3, np.float32))


def test_debug_firefly_elimination_known_answer():
    # k = 1: threshold 1.299; |0 - 0.75| = 0.75 kept, |3 - 0.75| = 2.25 dropped
    s = _intensity_samples([0, 0, 0, 3])
    np.testing.assert_array_equal(orc.resolve_pixel(s, True, 1.0, debug_mode=22), np.float32([1, 1, 1]))
    # k = 2 keeps all four samples
    np.testing.assert_array_equal(orc.resolve_pixel(s, True, 2.0, debug_mode=22), np.zeros(3, np.float32))
    # ten samples, two far outliers: intensities 8 x 1, 2 x 21 -> mean 5, sigma 8, k = 1 drops both
    s = _intensity_samples([1] * 8 + [21, 21])
    np.testing.assert_array_equal(orc.resolve_pixel(s, True, 1.0, debug_mode=22), np.float32([2, 2, 2]))


def test_debug_clamp_modes_without_the_clamp_average_the_samples():
    # with the clamp off CleanupFireflies is never called (Tracer.cpp:595-596)
    s = _intensity_samples([0, 0, 0, 3])
    mean = s.astype(np.float64).mean(axis=0)
    for mode in (21, 22):
        np.testing.assert_allclose(orc.resolve_pixel(s, False, 1.0, debug_mode=mode), mean, rtol=1e-6)


def test_firefly_clamp_all_rejected_divides_by_one():
    # zero variance: |I - mean| > 0 is false for all, nothing rejected
    s = np.full((8, 3), 0.25, dtype=np.float32)
    np.testing.assert_allclose(orc.resolve_pixel(s, True, 0.0), [0.25] * 3, rtol=1e-7)


# --------------------------------------------------------------------------- BVH
def soup(n, seed):
    rng = np.random.default_rng(seed)
    c = rng.uniform(-5, 5, (n, 1, 3))
    return (c + rng.normal(scale=0.3, size=(n, 3, 3))).astype(np.float32)


def meshes():
    sph = mt.scenes.uv_sphere(0.45).positions
    terr = mt.scenes.large_scene(terrain_n=48, num_spheres=50, tex_size=16)[0]
    return {"sphere": sph, "soup": soup(3000, 4), "terrain": terr.meshes[0].positions,
            "icospheres": terr.meshes[1].positions}


def check_bvh_invariants(pos, nodes, idx, max_tri, max_depth):
    T = pos.shape[0]
    f = nodes.view(np.float32)
    lo = pos.reshape(-1, 3).min(0)
    hi = pos.reshape(-1, 3).max(0)
    np.testing.assert_array_equal(f[0, 0:3], lo)
    np.testing.assert_array_equal(f[0, 3:6], hi)
    seen = np.zeros(T, dtype=bool)
    stack = [(0, 0)]
    max_d = 0
    while stack:
        ni, d = stack.pop()
        max_d = max(max_d, d)
        a, b = int(nodes[ni, 6]), int(nodes[ni, 7])
        if a & A.MT_BVH_LEAF_BIT:
            first = a & ~A.MT_BVH_LEAF_BIT
            seen[idx[first:first + b]] = True
            continue
        assert b == a + 1, "siblings must be adjacent"
        # children: parent box clipped on exactly one axis at the same plane
        pa, pb = f[ni, 0:6], (f[a, 0:6], f[b, 0:6])
        diff_a = np.nonzero(pb[0] != pa)[0]
        diff_b = np.nonzero(pb[1] != pa)[0]
        assert len(diff_a) <= 1 and len(diff_b) <= 1
        if len(diff_a) == 1:
            assert diff_a[0] >= 3 and (len(diff_b) == 0 or diff_b[0] == diff_a[0] - 3)
        stack += [(a, d + 1), (b, d + 1)]
    assert seen.all(), "every triangle must be reachable"
    assert max_d <= max(1, max_depth - 1) or max_depth < 2


@pytest.mark.parametrize("name", ["sphere", "soup", "terrain", "icospheres"])
@pytest.mark.parametrize("max_tri,max_depth", [(32, 32), (8, 32), (4, 12), (2, 64)])
def test_product_builder_equals_oracle_builder(name, max_tri, max_depth):
    pos = meshes()[name]
    n1, i1 = orc.bvh_build(pos, max_tri, max_depth)
    n2, i2 = mt.bvh_build(pos, max_tri, max_depth)
    # node 1 is never written by the reference (BVH.cpp:265-266); compare the rest
    np.testing.assert_array_equal(n1[0], n2[0])
    np.testing.assert_array_equal(n1[2:], n2[2:])
    np.testing.assert_array_equal(i1, i2)
    check_bvh_invariants(pos, n1, i1, max_tri, max_depth)


def test_builder_unsigned_depth_wrap_matches():
    # bvhMaxDepth 1 wraps the unsigned depth budget (Mesh.cpp:40, BVH.cpp:211)
    pos = soup(500, 9)
    n1, i1 = orc.bvh_build(pos, 4, 1)
    n2, i2 = mt.bvh_build(pos, 4, 1)
    np.testing.assert_array_equal(n1[2:], n2[2:])
    np.testing.assert_array_equal(i1, i2)


def test_builder_rejects_empty_and_unsplittable():
    same = np.zeros((40, 3, 3), dtype=np.float32) + np.float32([[0, 0, 0], [1, 0, 0], [0, 1, 0]])
    for pos in (np.zeros((0, 3, 3), dtype=np.float32), same):
        with pytest.raises(RuntimeError):
            orc.bvh_build(pos, 32, 32)
        with pytest.raises(mt.MTError):
            mt.bvh_build(pos, 32, 32)


def test_oracle_bounce_sampling_branches():
    """The oracle's bounce sample with given uniforms: u[0] above the specular
    probability picks the cosine lobe, whose direction and pdf follow
    cosine_hemisphere; a GGX sample that reflects below the surface falls back."""
    q = np.zeros((3, 16), np.float32)
    q[:, 0:3] = [0.0, 1.0, 0.0]        # V
    q[:, 3:6] = [0.0, 1.0, 0.0]        # N
    q[:, 6:9] = 0.5
    q[:, 9] = 0.5
    q[:, 10] = 0.0
    q[0, 11:16] = [0.999, 0.0, 0.25, 0.5, 0.5]   # cosine lobe, u1 = 0: straight up
    q[1, 11:16] = [0.0, 0.3, 0.7, 0.5, 0.5]      # GGX lobe
    q[2, 11:16] = [0.0, 0.999999, 0.1, 0.25, 0.5]  # GGX at grazing V? (V = N: reflection stays above)
    r = orc.brdf_sample(q)
    lobes = r[:, 5].view(np.int32)
    assert lobes[0] == 0 and lobes[1] == 1
    assert r[0, 1] > 0.99 and r[0, 3] > 0.0
    assert np.all(np.abs(np.linalg.norm(r[:, 0:3], axis=1) - 1) < 1e-5)
    assert np.all(r[:, 4] >= 0.05) and np.all(r[:, 4] <= 0.95)
