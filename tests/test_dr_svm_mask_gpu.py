"""GPU: SVM border sampling (CastBorderRaySVM, diff_render/MultiRendererDR.cpp:
1651-1931) and the ray-casting mask (:369-383, :443-448, :1097-1100, :1164-1167)
against the oracle.

SVM: every classification ray, the SVM fit and the sampling line are the same
float operations on both sides, and the stripe samples come from the same hash,
so the view's gradient equals the oracle's within the gradient bar (1e-3 of its
norm; atomics sum in another order) and differs from random border sampling's.
Mask: a pixel's hit or miss is bit-exact, so the masks after every step equal the
oracle's byte for byte, and the step gradients agree within the same bar."""
import numpy as np
import pytest

from litert_gb300 import dr, lrt, scenes
from oracle import oracle as orc
from oracle import oracle_dr as od

pytestmark = pytest.mark.gpu

S = 48


def _setup(**kw):
    up = scenes.union_params()
    sdf_t = lrt.Sdf(up["spheres"], up["boxes"], up["k"])
    hdr, nodes, values, target = dr.grid_sbs(6, 4, sdf_t, None)
    _, _, _, init = dr.grid_sbs(6, 4, lrt.Sdf(spheres=np.array([[0, 0, 0, 0.55]], np.float32)), [0.8, 0.3, 0.2])
    pj = lrt.perspective(45.0, 1.0, 0.01, 100.0)
    views = [(S, S, lrt.look_at([2.6 * np.sin(a), 1.0, 2.6 * np.cos(a)], [0, 0, 0], [0, 1, 0]), pj)
             for a in (0.3, 2.0)]
    R = dr.MultiRendererDR()
    R.SetScene(hdr, nodes, values, target)
    R.SetReference([np.zeros((S, S, 4), np.float32)] * 2, [v[2] for v in views], [v[3] for v in views])
    R.SetPreset(dr.default_preset(reconstruction_flags=0, border_spp=0))
    imgs = []
    for i in range(2):
        R.render_grad(i)
        imgs.append(R.getLastImage(i).copy())
    R.set_params(init)
    R.SetReference(imgs, [v[2] for v in views], [v[3] for v in views])
    preset = dr.default_preset(seed=3, accumulate_batch=1, **kw)
    R.SetPreset(preset)
    osc = od.DrScene(orc.SbsHeader(hdr.brick_size, hdr.brick_pad, hdr.bytes_per_value, hdr.aux_data), nodes, values,
                     init.size, pairs=R.bvh2())
    lights = [(preset.lights[i].type, np.array(preset.lights[i].dir[:], np.float32),
               np.array(preset.lights[i].color[:], np.float32)) for i in range(preset.n_lights)]
    op = od.make_preset(render_mode=preset.render_mode, reconstruction=preset.reconstruction_flags,
                        border_spp=preset.border_spp, seed=preset.seed, lights=lights, lr=preset.opt_lr,
                        accumulate_batch=1, spp=preset.spp, border_relax_eps=preset.border_relax_eps,
                        border_sampling=preset.border_sampling, raycasting_mask=preset.raycasting_mask)
    oviews = [od.make_view(v[0], v[1], v[2], v[3], lrt.inverse4x4) for v in views]
    return R, osc, init, op, oviews, imgs


@pytest.mark.parametrize("border_spp", [16, 64, 256])
def test_svm_border_gradient_matches_oracle(border_spp):
    R, osc, init, op, oviews, imgs = _setup(border_spp=border_spp, border_sampling=1, border_relax_eps=0.01)
    _, g = R.render_grad(0)
    o = osc.render(init, op, oviews[0], imgs[0].reshape(-1, 4), threads=1)
    nrm = np.linalg.norm(o["grad"])
    assert nrm > 0
    assert np.linalg.norm(g - o["grad"]) <= 1e-3 * nrm
    # the border integral is part of it, and differs from random sampling's
    R.SetPreset(dr.default_preset(seed=3, accumulate_batch=1, border_spp=border_spp, border_relax_eps=0.01))
    _, g_rand = R.render_grad(0)
    R.SetPreset(dr.default_preset(seed=3, accumulate_batch=1, border_spp=0))
    _, g_none = R.render_grad(0)
    assert np.linalg.norm(g - g_none) > 1e-3 * nrm
    assert np.linalg.norm(g - g_rand) > 1e-3 * nrm
    R.close()


def test_svm_rejects_too_many_border_samples():
    R, *_ = _setup(border_spp=16)
    with pytest.raises(lrt.LrtError):
        R.SetPreset(dr.default_preset(border_spp=2048, border_sampling=1))
    R.close()


@pytest.mark.parametrize("spp,sampling", [(1, 0), (4, 0), (1, 1)])
def test_raycasting_mask_matches_oracle_over_steps(spp, sampling):
    R, osc, init, op, oviews, imgs = _setup(border_spp=16, raycasting_mask=1, opt_lr=0.02, spp=spp,
                                            border_sampling=sampling)
    masks = [np.ones(S * S, np.uint8) for _ in oviews]
    params = init.copy()
    state = np.zeros(2 * params.size, np.float32)
    shrank = False
    for it in range(3):
        R.step(it)
        o = osc.step(params, op, oviews, imgs, it, state, threads=1, masks=masks)
        for v in range(2):
            got = R.get(dr.GET_CAST_MASK, v)
            assert np.array_equal(got, masks[v]), (it, v, int((got != masks[v]).sum()))
            shrank |= bool(masks[v].sum() < S * S)
        g = R.get(dr.GET_GRAD)
        want = o["grad"] * 2      # the engine's buffer holds the batch sum, before the division
        assert np.linalg.norm(g - want) <= 1e-3 * np.linalg.norm(want)
        # keep both sides on the same parameters: the next step starts from the oracle's
        R.set_params(params)
    assert shrank
    R.close()


@pytest.mark.parametrize("case", ["away", "one_pixel", "ragged"])
def test_dr_edge_views_match_oracle(case):
    """RenderDR on a view that sees nothing (loss from the reference image alone, no
    gradient), a one-pixel view and a ragged 13 x 7 view: image, loss and gradient
    against the oracle."""
    up = scenes.union_params()
    hdr, nodes, values, target = dr.grid_sbs(6, 4, lrt.Sdf(up["spheres"], up["boxes"], up["k"]), None)
    _, _, _, init = dr.grid_sbs(6, 4, lrt.Sdf(spheres=np.array([[0, 0, 0, 0.55]], np.float32)), [0.8, 0.3, 0.2])
    if case == "away":
        w, h, eye, at = 24, 16, [0, 0, 2.6], [0, 0, 6]
    elif case == "one_pixel":
        w, h, eye, at = 1, 1, [0.05, 0.02, 2.6], [0, 0, 0]
    else:
        w, h, eye, at = 13, 7, [1.5, 1.0, 2.2], [0, 0, 0]
    wv, pj = lrt.look_at(eye, at, [0, 1, 0]), lrt.perspective(45.0, float(w) / h, 0.01, 100.0)
    ref = np.random.default_rng(5).uniform(0, 1, (h, w, 4)).astype(np.float32)
    R = dr.MultiRendererDR()
    R.SetScene(hdr, nodes, values, init)
    R.SetReference([ref], [wv], [pj])
    preset = dr.default_preset(seed=3, border_spp=32)
    R.SetPreset(preset)
    loss, g = R.render_grad(0)
    img = R.getLastImage(0).reshape(-1, 4)
    osc = od.DrScene(orc.SbsHeader(hdr.brick_size, hdr.brick_pad, hdr.bytes_per_value, hdr.aux_data), nodes, values,
                     init.size, pairs=R.bvh2())
    lights = [(preset.lights[i].type, np.array(preset.lights[i].dir[:], np.float32),
               np.array(preset.lights[i].color[:], np.float32)) for i in range(preset.n_lights)]
    op = od.make_preset(render_mode=preset.render_mode, reconstruction=preset.reconstruction_flags, border_spp=32,
                        seed=3, lights=lights, lr=preset.opt_lr)
    o = osc.render(init, op, od.make_view(w, h, wv, pj, lrt.inverse4x4), ref.reshape(-1, 4), threads=1)
    R.close()
    assert np.array_equal(img.view(np.uint32), o["image"].view(np.uint32))
    assert abs(loss - o["loss"]) <= 1e-9 * max(1.0, abs(o["loss"]))
    if case == "away":
        assert not np.any(img[:, 3]) and not np.any(g) and not np.any(o["grad"])
    else:
        nrm = np.linalg.norm(o["grad"])
        assert np.linalg.norm(g - o["grad"]) <= 1e-3 * max(nrm, 1e-30)
