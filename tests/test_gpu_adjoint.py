"""The path-replay adjoint on the GPU (mt_render_grad, through the C ABI).

1. Against the oracle's CPU replay gradient (same convention, same counter
   RNG, independent implementation): material base colour / roughness /
   metallic, light intensity and albedo-texel gradients agree to 1e-2 in norm
   and per large component.
2. Against central finite differences (h = 1e-3) of the GPU forward render on
   32 parameters (base colours, light intensities, albedo texels), with the
   energy cut-off and firefly clamp off so the estimator is smooth in them:
   <= 1e-2 relative; and on 16 roughness and metallic factors with one bounce,
   where they enter a sample only through the BRDF evaluation.
3. The loss it reports equals sum (image - target)^2 of the image it renders,
   and that image equals mt_render_device's.
4. A torch.autograd.Function (this harness only) backpropagates through it.
"""
import numpy as np
import pytest

import mitrace_gb300 as mt
from mitrace_gb300 import _abi as A
from oracle import oracle_py as orc

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def gpu_grad(scene, cfg, target):
    nm, nl = len(scene.materials), len(scene.lights)
    nt = mt.scenes.num_grad_texels(scene)
    dev = "cuda"
    t = torch.from_numpy(np.ascontiguousarray(target, np.float32)).to(dev)
    out = {
        "image": torch.zeros((cfg.height, cfg.width, 3), device=dev),
        "loss": torch.zeros(1, device=dev),
        "d_base": torch.zeros((nm, 3), device=dev),
        "d_roughness": torch.zeros(nm, device=dev),
        "d_metallic": torch.zeros(nm, device=dev),
        "d_light": torch.zeros(max(nl, 1), device=dev),
        "d_texels": torch.zeros(max(nt, 1), device=dev),
    }
    with mt.Tracer(scene, cfg) as tr:
        tr.render_grad_device(t.data_ptr(), out["image"].data_ptr(), out["loss"].data_ptr(),
                              out["d_base"].data_ptr(), out["d_roughness"].data_ptr(),
                              out["d_metallic"].data_ptr(), out["d_light"].data_ptr(),
                              out["d_texels"].data_ptr() if nt else 0, torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
    r = {k: v.cpu().numpy() for k, v in out.items()}
    r["loss"] = float(r["loss"][0])
    r["d_light"] = r["d_light"][:nl]
    r["d_texels"] = r["d_texels"][:nt]
    return r


def gpu_image(scene, cfg):
    out = torch.zeros((cfg.height, cfg.width, 3), device="cuda")
    with mt.Tracer(scene, cfg) as tr:
        tr.render_device(out.data_ptr(), torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
    return out.cpu().numpy()


def grid_case():
    """Adjoint scene with roughness from 0.25: at roughness 0.05 the GGX lobe
    (alpha^2 = 0.0025) makes dD/droughness so steep that a one-ulp difference
    in a sampled direction (GPU vs host sinf/cosf) moves single samples'
    roughness gradients by percent; the other parameters are unaffected and
    the 0.05 spheres stay in the finite-difference test."""
    scene, cfg = mt.scenes.adjoint_scene(width=96, height=96, samples=4, texture_size=64)
    for k, m in enumerate(scene.materials[:49]):
        m.roughness = 0.25 + 0.75 * (k % 7) / 6.0
    return scene, cfg


CASES = {
    "box_room": lambda: mt.box_room(width=64, height=64, samples=8, seed=2),
    "material_grid": grid_case,
}


def close(g, o, name):
    g, o = np.asarray(g, np.float64).ravel(), np.asarray(o, np.float64).ravel()
    if o.size == 0:
        return
    scale = np.abs(o).max()
    assert np.linalg.norm(g - o) <= 1e-2 * np.linalg.norm(o) + 1e-6, f"{name}: norm"
    big = np.abs(o) > 0.05 * scale
    assert np.all(np.abs(g[big] - o[big]) <= 2e-2 * np.abs(o[big])), f"{name}: components"


@pytest.mark.parametrize("name", list(CASES))
def test_gpu_adjoint_matches_cpu_replay(name):
    scene, cfg = CASES[name]()
    rng = np.random.default_rng(1)
    target = rng.uniform(0.2, 0.6, (cfg.height, cfg.width, 3)).astype(np.float32)
    g = gpu_grad(scene, cfg, target)
    o = orc.OracleScene(mt.PackedScene(scene), cfg).render_grad(target, mt.scenes.num_grad_texels(scene))
    assert abs(g["loss"] - o["loss"]) <= 1e-3 * o["loss"]
    for k in ("d_base", "d_roughness", "d_metallic", "d_light", "d_texels"):
        close(g[k], o[k], f"{name} {k}")


def test_loss_and_image_are_consistent():
    scene, cfg = CASES["box_room"]()
    target = np.full((cfg.height, cfg.width, 3), 0.25, np.float32)
    g = gpu_grad(scene, cfg, target)
    img = gpu_image(scene, cfg)
    np.testing.assert_array_equal(g["image"], img)
    assert abs(g["loss"] - float(((img.astype(np.float64) - target) ** 2).sum())) <= 1e-4 * g["loss"]


def fd_scene():
    scene, cfg = mt.scenes.adjoint_scene(width=96, height=96, samples=16, texture_size=32, seed=5)
    for m in scene.materials:  # metallic 0: the lobe choice does not depend on the base colour
        m.metallic = 0.0
    scene.lights = scene.lights[:1]  # one light: the reservoir pick does not depend on intensities
    cfg.terminate_energy = 0.0
    cfg.firefly_enable = 0
    return scene, cfg


def test_gpu_adjoint_matches_finite_differences():
    h = 1e-3
    scene, cfg = fd_scene()
    target = np.full((cfg.height, cfg.width, 3), 0.2, np.float32)
    g = gpu_grad(scene, cfg, target)
    rng = np.random.default_rng(7)
    # 32 parameters: base colours of visible materials, both lights, ground texels
    nz = [(m, c) for m in range(len(scene.materials)) for c in range(3) if abs(g["d_base"][m, c]) > 1e-2]
    picks = [("base", *nz[i]) for i in rng.choice(len(nz), size=min(20, len(nz)), replace=False)]
    picks += [("light", 0)]
    tex_nz = np.nonzero(np.abs(g["d_texels"]) > 1e-2 * np.abs(g["d_texels"]).max())[0]
    picks += [("texel", int(i)) for i in rng.choice(tex_nz, size=32 - len(picks), replace=False)]

    def loss_with(kind, idx, s):
        sc, cf = fd_scene()
        if kind == "base":
            m, c = idx
            b = list(sc.materials[m].base_color)
            b[c] += s * h
            sc.materials[m].base_color = tuple(b)
        elif kind == "light":
            sc.lights[idx[0]].color = tuple(np.float32(sc.lights[idx[0]].color) * np.float32(1 + s * h))
        else:
            tex = sc.textures[sc.materials[49].base_tex].rgb32f
            tex.reshape(-1)[idx[0]] += s * h
        img = gpu_image(sc, cf).astype(np.float64)
        return float(((img - target) ** 2).sum())

    worst = 0.0
    for kind, *idx in picks:
        fd = (loss_with(kind, idx, 1) - loss_with(kind, idx, -1)) / (2 * h)
        ad = {"base": lambda: g["d_base"][idx[0], idx[1]], "light": lambda: g["d_light"][idx[0]],
              "texel": lambda: g["d_texels"][idx[0]]}[kind]()
        rel = abs(fd - ad) / max(abs(fd), 1e-6)
        worst = max(worst, rel)
        assert rel <= 1e-2, (kind, idx, fd, ad)
    assert len(picks) == 32


def fd_scene_one_bounce():
    """bounces = 1: a sample is the primary vertex's emission plus its
    next-event estimate (or the sky on a miss); the bounce direction it samples
    is never traced.  Roughness and metallic then enter the sample only through
    EvaluateBRDF of the light direction, so holding the sampling decisions
    fixed (the path-replay convention) and moving the parameters in the forward
    render change the sample in the same way, and central differences pin
    their gradients.  With more bounces the GGX-sampled direction moves with
    roughness (and the lobe choice with metallic): the two then agree only in
    expectation."""
    scene, cfg = fd_scene()
    cfg.bounces = 1
    for j in range(7):  # metallic inside (0, 1): away from clamp(metallic, 0, 1)'s kinks
        for i in range(7):
            scene.materials[j * 7 + i].metallic = 0.1 + 0.8 * j / 6.0
    return scene, cfg


def test_gpu_adjoint_roughness_and_metallic_match_finite_differences():
    h = 1e-3
    scene, cfg = fd_scene_one_bounce()
    target = np.full((cfg.height, cfg.width, 3), 0.2, np.float32)
    g = gpu_grad(scene, cfg, target)
    rng = np.random.default_rng(9)
    # spheres of columns 1..6 (roughness 0.21 .. 1, above the 0.05 floor of BRDF.hpp)
    cand = [m for m in range(49) if m % 7 > 0]
    picks = []
    for kind, key in (("rough", "d_roughness"), ("metal", "d_metallic")):
        nz = [m for m in cand if abs(g[key][m]) > 1e-2 * np.abs(g[key]).max()]
        picks += [(kind, int(m)) for m in rng.choice(nz, size=min(8, len(nz)), replace=False)]

    def loss_with(kind, m, s):
        sc, cf = fd_scene_one_bounce()
        if kind == "rough":
            sc.materials[m].roughness += s * h
        else:
            sc.materials[m].metallic += s * h
        img = gpu_image(sc, cf).astype(np.float64)
        return float(((img - target) ** 2).sum())

    for kind, m in picks:
        fd = (loss_with(kind, m, 1) - loss_with(kind, m, -1)) / (2 * h)
        ad = float(g["d_roughness" if kind == "rough" else "d_metallic"][m])
        assert abs(fd - ad) <= 1e-2 * max(abs(fd), 1e-6), (kind, m, fd, ad)
    assert len(picks) == 16


class RenderLoss(torch.autograd.Function):
    """loss(base colours of all materials) with the adjoint as its backward;
    exists only in this test harness."""

    @staticmethod
    def forward(ctx, base, scene, cfg, target):
        sc = scene
        for m, b in zip(sc.materials, base.detach().cpu().numpy()):
            m.base_color = (float(b[0]), float(b[1]), float(b[2]), 1.0)
        g = gpu_grad(sc, cfg, target)
        ctx.save_for_backward(torch.from_numpy(g["d_base"]))
        return torch.tensor(g["loss"], dtype=torch.float64)

    @staticmethod
    def backward(ctx, grad_out):
        (d_base,) = ctx.saved_tensors
        return grad_out * d_base.to(torch.float64), None, None, None


def test_autograd_function_backpropagates():
    scene, cfg = CASES["box_room"]()
    target = np.full((cfg.height, cfg.width, 3), 0.25, np.float32)
    base = torch.tensor([m.base_color[:3] for m in scene.materials], dtype=torch.float64, requires_grad=True)
    loss = RenderLoss.apply(base, scene, cfg, target)
    loss.backward()
    g = gpu_grad(scene, cfg, target)
    # a second run of the adjoint: its float atomic sums add in a scheduling-
    # dependent order, so the two agree to rounding (measured up to ~1.1e-6
    # relative), not bit for bit
    np.testing.assert_allclose(base.grad.numpy(), g["d_base"], rtol=1e-5)
    assert np.abs(base.grad.numpy()).max() > 0


def test_image_gradient_input_equals_l2_target_form():
    """mt_render_grad with d_image = 2 (image - target) gives the same gradient
    as the L2-loss form (any loss's image gradient can be supplied)."""
    scene, cfg = CASES["box_room"]()
    target = np.full((cfg.height, cfg.width, 3), 0.3, np.float32)
    g = gpu_grad(scene, cfg, target)
    nm, nl = len(scene.materials), len(scene.lights)
    dimg = torch.from_numpy(2.0 * (g["image"] - target)).cuda()
    out = {k: torch.zeros(v, device="cuda") for k, v in
           (("image", cfg.height * cfg.width * 3), ("d_base", nm * 3), ("d_roughness", nm), ("d_metallic", nm),
            ("d_light", max(nl, 1)))}
    with mt.Tracer(scene, cfg) as tr:
        tr.render_grad_device(0, out["image"].data_ptr(), 0, out["d_base"].data_ptr(), out["d_roughness"].data_ptr(),
                              out["d_metallic"].data_ptr(), out["d_light"].data_ptr(), 0,
                              torch.cuda.current_stream().cuda_stream, d_image_ptr=dimg.data_ptr())
        torch.cuda.synchronize()
    # equal up to the order of the atomic sums
    np.testing.assert_allclose(out["d_base"].cpu().numpy().reshape(nm, 3), g["d_base"], rtol=1e-4, atol=1e-6)
    np.testing.assert_allclose(out["d_roughness"].cpu().numpy(), g["d_roughness"], rtol=1e-4, atol=1e-6)
    np.testing.assert_allclose(out["d_light"].cpu().numpy()[:nl], g["d_light"], rtol=1e-4, atol=1e-6)


def test_inverse_materials_descend_toward_hidden_colours():
    """The inverse-materials loop: hidden sphere base colours render a target;
    Adam on the base colours from grey, one handle for the whole loop
    (mt_update_materials between mt_render_grad calls), lowers the image loss
    and moves the colours toward the hidden ones."""
    scene, cfg = mt.scenes.adjoint_scene(width=64, height=64, samples=16, texture_size=32, seed=3)
    rng = np.random.default_rng(11)
    hidden = rng.uniform(0.2, 0.9, (49, 3)).astype(np.float32)
    for k in range(49):
        scene.materials[k].base_color = (*map(float, hidden[k]), 1.0)
    tscene, tcfg = mt.scenes.adjoint_scene(width=64, height=64, samples=256, texture_size=32, seed=3)
    tscene.materials = scene.materials
    target = gpu_image(tscene, tcfg)
    x = np.full((49, 3), 0.5, np.float32)
    for k in range(49):
        scene.materials[k].base_color = (0.5, 0.5, 0.5, 1.0)
    nm, nl = len(scene.materials), len(scene.lights)
    t = torch.from_numpy(target).cuda()
    bufs = {k: torch.zeros(v, device="cuda") for k, v in
            (("image", 64 * 64 * 3), ("loss", 1), ("d_base", nm * 3), ("d_roughness", nm), ("d_metallic", nm),
             ("d_light", max(nl, 1)))}
    m = np.zeros_like(x)
    v = np.zeros_like(x)
    losses = []
    err0 = float(np.abs(x - hidden).mean())
    with mt.Tracer(scene, cfg) as tr:
        for it in range(1, 31):
            for b in bufs.values():
                b.zero_()
            tr.render_grad_device(t.data_ptr(), bufs["image"].data_ptr(), bufs["loss"].data_ptr(),
                                  bufs["d_base"].data_ptr(), bufs["d_roughness"].data_ptr(),
                                  bufs["d_metallic"].data_ptr(), bufs["d_light"].data_ptr(), 0,
                                  torch.cuda.current_stream().cuda_stream)
            torch.cuda.synchronize()
            losses.append(float(bufs["loss"].item()))
            g = bufs["d_base"].cpu().numpy().reshape(nm, 3)[:49]
            m = 0.9 * m + 0.1 * g
            v = 0.999 * v + 0.001 * g * g
            x = np.clip(x - 0.03 * (m / (1 - 0.9 ** it)) / (np.sqrt(v / (1 - 0.999 ** it)) + 1e-8), 0.0, 1.0)
            for k in range(49):
                scene.materials[k].base_color = (*map(float, x[k]), 1.0)
            tr.update_materials(scene.materials)
    assert losses[-1] < 0.35 * losses[0], losses
    assert float(np.abs(x - hidden).mean()) < 0.6 * err0

