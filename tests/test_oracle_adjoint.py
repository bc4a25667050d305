"""The oracle's path-replay gradient against central finite differences of its
own (deterministic, counter-RNG) forward render.  With the energy cut-off and
the firefly clamp disabled the estimator is smooth in the base colours and the
light intensity of the box room (metallic 0: the lobe choice does not depend
on the base colour), so the two must agree closely.  With the cut-off on, a
path whose throughput crosses the threshold jumps; the adjoint holds the
cut-off constant by design, and that case is asserted as such."""
import numpy as np
import pytest

import mitrace_gb300 as mt
from oracle import oracle_py as orc

H = 1e-3


def make(cutoff=False, clamp=False):
    sc, cf = mt.box_room(width=16, height=16, samples=4, seed=3)
    cf.firefly_enable = int(clamp)
    cf.terminate_energy = 0.1 if cutoff else 0.0
    return sc, cf


def loss_of(mod, cutoff=False, clamp=False, target=None):
    sc, cf = make(cutoff, clamp)
    mod(sc)
    img, _, _ = orc.OracleScene(mt.PackedScene(sc), cf).render(orc.RNG_COUNTER)
    return float(((img.astype(np.float64) - target) ** 2).sum())


def base_mod(m, c, s):
    def f(sc):
        b = list(sc.materials[m].base_color)
        b[c] += s * H
        sc.materials[m].base_color = tuple(b)
    return f


def light_mod(s):
    def f(sc):
        sc.lights[0].color = tuple(np.float32(sc.lights[0].color) * np.float32(1 + s * H))
    return f


def test_replay_gradient_matches_central_differences():
    target = np.full((16, 16, 3), 0.3, np.float32)
    sc, cf = make()
    g = orc.OracleScene(mt.PackedScene(sc), cf).render_grad(target)
    for m in range(3):
        for c in range(3):
            fd = (loss_of(base_mod(m, c, 1), target=target) - loss_of(base_mod(m, c, -1), target=target)) / (2 * H)
            assert abs(fd - g["d_base"][m, c]) <= 1e-3 * abs(fd), (m, c, fd, g["d_base"][m, c])
    fd = (loss_of(light_mod(1), target=target) - loss_of(light_mod(-1), target=target)) / (2 * H)
    assert abs(fd - g["d_light"][0]) <= 1e-3 * abs(fd)


def test_loss_and_image_match_forward_render():
    target = np.full((16, 16, 3), 0.3, np.float32)
    sc, cf = make(cutoff=True, clamp=True)
    o = orc.OracleScene(mt.PackedScene(sc), cf)
    g = o.render_grad(target)
    img, _, _ = o.render(orc.RNG_COUNTER)
    np.testing.assert_array_equal(g["image"], img)
    assert abs(g["loss"] - float(((img.astype(np.float64) - target) ** 2).sum())) <= 1e-4 * g["loss"]
