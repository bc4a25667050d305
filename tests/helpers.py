"""Shared helpers for the parity tests (CPU oracle vs the CUDA path)."""
import numpy as np

import mitrace_gb300 as mt
from oracle import oracle_py as orc


def small_grid(width=96, height=54, samples=8, seed=3, segments=64, rings=32):
    return mt.scenes.material_grid(width=width, height=height, samples=samples, seed=seed, segments=segments,
                                   rings=rings)


def many_instances(width=64, height=36, samples=4, seed=4, n=12):
    """The material grid's sphere and ground with n x n sphere instances at
    staggered depths (n * n + 1 instances: more than one 64-instance chunk of
    the world-box test, boxes overlapping along most rays)."""
    scene, cfg = small_grid(width=width, height=height, samples=samples, seed=seed, segments=16, rings=8)
    inst = []
    for j in range(n):
        for i in range(n):
            z = -0.5 * ((7 * i + 3 * j) % 4)
            inst.append(mt.scenes.InstanceData(0, (j * n + i) % 49,
                                               mt.scenes.translate((i - (n - 1) / 2) * 0.8, 0.45 + j * 0.8, z)))
    inst.append(mt.scenes.InstanceData(1, 49))
    scene.instances = inst
    return scene, cfg


def small_large_scene(width=64, height=36, samples=4, seed=5):
    return mt.scenes.large_scene(terrain_n=96, num_spheres=400, tex_size=128, width=width, height=height,
                                 samples=samples, seed=seed)


def scene_rays(scene, cfg, n, seed=0, tmax_range=None):
    """Half incoherent rays in the scene bounds, half camera rays."""
    lo, hi = mt.scene_bounds(scene)
    pad = 0.05 * (hi - lo)
    rng = np.random.default_rng(seed)
    r1 = mt.incoherent_rays(lo - pad, hi + pad, n - n // 2, seed=seed)
    o = orc.OracleScene(mt.PackedScene(scene), cfg)
    uv = rng.random((n // 2, 2)).astype(np.float32)
    r2 = o.camera_rays(uv)
    r = np.concatenate([r1, r2]).astype(np.float32)
    if tmax_range is not None:
        r[:, 3] = rng.uniform(tmax_range[0], tmax_range[1], r.shape[0]).astype(np.float32)
    return r


def as_f32(hits):
    return hits.view(np.float32)
