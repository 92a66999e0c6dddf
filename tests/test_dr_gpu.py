"""GPU: the differentiable render (dr_pixel / dr_border / dr_adam kernels)
against the CPU oracle, which is pinned to the reference's diff_render/BVH2DR.cpp.

Per view: the rendered image, the depth-discontinuity thresholds and the border
mask equal the oracle bit for bit; the loss agrees to 1e-9 relative (double
sums in another order); the gradient dLoss/dparams (interior + border integral,
getBaseGradientMult applied) agrees within 1e-3 relative in norm and per
component relative to the largest component, as the reference-gradient bar
asks (atomics sum in another order than the reference's per-thread slices).
Also: the interior gradient against double-precision central finite
differences, the optimisation iteration (batch handling + Adam) against the
oracle, a reconstruction that lowers the loss, and host-side rejections.
"""
import numpy as np
import pytest

from litert_gb300 import dr, lrt, scenes
from oracle import oracle as orc
from oracle import oracle_dr as od

pytestmark = pytest.mark.gpu

REL = 1e-3


def _problem(bc=6, bs=4, w=64, h=64, n_views=1, layout_in=True):
    up = scenes.union_params()
    sdf_t = lrt.Sdf(up["spheres"], up["boxes"], up["k"])
    hdr, nodes, values, target = dr.grid_sbs(bc, bs, sdf_t, None)
    _, _, _, init = dr.grid_sbs(bc, bs, lrt.Sdf(spheres=np.array([[0, 0, 0, 0.55]], np.float32)), [0.8, 0.3, 0.2])
    if not layout_in:
        hdr = lrt.SbsHeader(hdr.brick_size, hdr.brick_pad, hdr.bytes_per_value, lrt.SBS_LAYOUT_ID32F_IRGB32F)
    pj = lrt.perspective(45.0, w / h, 0.01, 100.0)
    views = []
    for i in range(n_views):
        a = 2 * np.pi * i / max(n_views, 1) + 0.3
        wv = lrt.look_at([2.6 * np.sin(a), 1.0, 2.6 * np.cos(a)], [0, 0, 0], [0, 1, 0])
        views.append((w, h, wv, pj))
    return hdr, nodes, values, target, init, views


def _oracle(hdr, nodes, values, params, pairs, need_normal=True):
    return od.DrScene(orc.SbsHeader(hdr.brick_size, hdr.brick_pad, hdr.bytes_per_value, hdr.aux_data), nodes, values,
                      params.size, pairs=pairs, need_normal=need_normal)


def _orc_preset(p):
    lights = [(p.lights[i].type, np.array(p.lights[i].dir[:], np.float32), np.array(p.lights[i].color[:], np.float32))
              for i in range(p.n_lights)]
    return od.make_preset(render_mode=p.render_mode, reconstruction=p.reconstruction_flags, input_type=p.input_type,
                          loss=p.loss_function, spp=p.spp, border_spp=p.border_spp, border_relax_eps=p.border_relax_eps,
                          seed=p.seed, lights=lights, lr=p.opt_lr, beta1=p.opt_beta_1, beta2=p.opt_beta_2,
                          eps=p.opt_eps, accumulate_batch=p.accumulate_batch, border_sampling=p.border_sampling)


def _targets(R, views, target_params, preset):
    """Target images: the target grid rendered by the same DR forward."""
    R.set_params(target_params)
    R.SetReference([np.zeros((v[1], v[0], 4), np.float32) for v in views], [v[2] for v in views], [v[3] for v in views])
    R.SetPreset(dr.default_preset(render_mode=preset.render_mode, spp=preset.spp, seed=preset.seed,
                                  reconstruction_flags=0, border_spp=0))
    imgs = []
    for i in range(len(views)):
        R.render_grad(i)
        imgs.append(R.getLastImage(i).copy())
    return imgs


def _check_grad(g, want):
    nrm = np.linalg.norm(want)
    assert nrm > 0
    assert np.linalg.norm(g - want) <= REL * nrm, (np.linalg.norm(g - want) / nrm)
    assert np.abs(g - want).max() <= REL * np.abs(want).max()


def _setup(preset, layout_in=True, spp_views=1, w=64, h=64):
    hdr, nodes, values, target, init, views = _problem(n_views=spp_views, w=w, h=h, layout_in=layout_in)
    R = dr.MultiRendererDR()
    R.SetScene(hdr, nodes, values, target)
    imgs = _targets(R, views, target, preset)
    R.set_params(init)
    R.SetReference(imgs, [v[2] for v in views], [v[3] for v in views])
    R.SetPreset(preset)
    osc = _oracle(hdr, nodes, values, init, R.bvh2(), need_normal=preset.render_mode in (1, 4))
    return R, osc, init, views, imgs


def _oview(v):
    return od.make_view(v[0], v[1], v[2], v[3], lrt.inverse4x4)


@pytest.mark.parametrize("cfg", [
    dict(),                                                     # Lambert, colour + geometry, border 64
    dict(warp_aggregate=0),
    dict(spp=4),
    dict(render_mode=dr.RENDER_DIFFUSE),
    dict(render_mode=dr.RENDER_NORMAL, reconstruction_flags=dr.RECON_GEOMETRY),
    dict(render_mode=dr.RENDER_MASK, reconstruction_flags=dr.RECON_GEOMETRY),
    dict(loss_function=1),
    dict(layout_in=False),
    dict(render_mode=dr.RENDER_LINEAR_DEPTH, input_type=1, reconstruction_flags=dr.RECON_GEOMETRY),
    # SVM border sampling (CastBorderRaySVM) across the render modes of the reference's test 4
    dict(border_sampling=1),
    dict(border_sampling=1, render_mode=dr.RENDER_DIFFUSE),
    dict(border_sampling=1, render_mode=dr.RENDER_MASK, reconstruction_flags=dr.RECON_GEOMETRY),
    dict(border_sampling=1, render_mode=dr.RENDER_LINEAR_DEPTH, input_type=1, reconstruction_flags=dr.RECON_GEOMETRY),
    dict(border_sampling=1, border_relax_eps=2e-4),
])
def test_render_grad_matches_oracle(cfg):
    cfg = dict(cfg)
    layout_in = cfg.pop("layout_in", True)
    preset = dr.default_preset(border_spp=64, seed=7, **cfg)
    R, osc, init, views, imgs = _setup(preset, layout_in=layout_in)
    loss, g = R.render_grad(0)
    o = osc.render(init, _orc_preset(preset), _oview(views[0]), imgs[0], threads=1)
    img = R.get(dr.GET_IMAGE, 0)
    assert (o["image"][:, 3] > 0).sum() > 300
    assert np.array_equal(img.view(np.uint32), o["image"].view(np.uint32))
    assert np.array_equal(R.get(dr.GET_DEPTH, 0).view(np.uint32), o["depth"].view(np.uint32))
    assert np.array_equal(R.get(dr.GET_BORDER, 0).astype(bool), o["border"])
    assert abs(loss - o["loss"]) <= 1e-9 * max(1.0, abs(o["loss"]))
    _check_grad(g, o["grad"])
    assert R.last_launch_count() >= 2
    R.close()


@pytest.mark.parametrize("sampling", [0, 1])
def test_border_integral_alone_matches_oracle(sampling):
    """The border term by itself (colour reconstruction off, interior geometry
    PDs cancelled by rendering with DNORM/DDIFFUSE only through the border), with
    random and with SVM border sampling."""
    preset = dr.default_preset(border_spp=128, seed=3, reconstruction_flags=dr.RECON_GEOMETRY, render_mode=dr.RENDER_MASK,
                               border_sampling=sampling)
    R, osc, init, views, imgs = _setup(preset)
    _, g = R.render_grad(0)
    o = osc.render(init, _orc_preset(preset), _oview(views[0]), imgs[0], threads=1)
    assert np.count_nonzero(o["grad"]) > 50      # MASK: every nonzero comes from the border integral
    _check_grad(g, o["grad"])
    R.close()


def test_interior_gradient_matches_f64_finite_differences():
    preset = dr.default_preset(border_spp=0, seed=5)
    R, osc, init, views, imgs = _setup(preset)
    _, g = R.render_grad(0)
    op = _orc_preset(preset)
    ov = _oview(views[0])
    N = ov.width * ov.height
    gm = np.float32((init.size + 1.0) ** (2.0 / 3.0) / N)
    nd = 25 ** 3
    P = init.astype(np.float64)
    _, hc0 = osc.loss_f64(P, op, ov, imgs[0])
    # colour parameters: exact up to rounding
    for i in (np.nonzero(g[nd:])[0][:25] + nd):
        P[i] += 1e-4
        lp, _ = osc.loss_f64(P, op, ov, imgs[0])
        P[i] -= 2e-4
        lm, _ = osc.loss_f64(P, op, ov, imgs[0])
        P[i] += 1e-4
        fd = (lp - lm) / 2e-4 * N * gm
        assert abs(g[i] - fd) <= 2e-4 * max(1.0, abs(fd)), (i, g[i], fd)
    # distance parameters where no pixel changes coverage: aggregate agreement
    errs, pairs = [], []
    for i in np.argsort(-np.abs(g[:nd]))[:50]:
        P[i] += 2e-5
        lp, hp = osc.loss_f64(P, op, ov, imgs[0])
        P[i] -= 4e-5
        lm, hm = osc.loss_f64(P, op, ov, imgs[0])
        P[i] += 2e-5
        if not (np.array_equal(hp, hc0) and np.array_equal(hm, hc0)):
            continue
        fd = (lp - lm) / 4e-5 * N * gm
        errs.append(abs(g[i] - fd) / max(abs(fd), 1e-3 * np.abs(g[:nd]).max()))
        pairs.append((g[i], fd))
    assert len(errs) >= 25
    a = np.array(pairs)
    assert np.median(errs) < 0.01 and np.percentile(errs, 90) < 0.1
    assert np.linalg.norm(a[:, 0] - a[:, 1]) / np.linalg.norm(a[:, 1]) < 0.25
    R.close()


@pytest.mark.parametrize("accumulate", [0, 1])
def test_optimisation_step_matches_oracle(accumulate):
    """One OptimizeFixedStructure iteration over 3 views: per-view losses, the
    batch gradient (the reference keeps only the last image's; accumulate sums
    them), Adam's moments and the updated parameters."""
    preset = dr.default_preset(border_spp=32, seed=11, opt_lr=3e-3, accumulate_batch=accumulate)
    hdr, nodes, values, target, init, views = _problem(n_views=3, w=48, h=48)
    R = dr.MultiRendererDR()
    R.SetScene(hdr, nodes, values, target)
    imgs = _targets(R, views, target, preset)
    R.set_params(init)
    R.SetReference(imgs, [v[2] for v in views], [v[3] for v in views])
    R.SetPreset(preset)
    osc = _oracle(hdr, nodes, values, init, R.bvh2())
    P = init.copy()
    st = np.zeros(2 * P.size, np.float32)
    losses = R.step(0)
    o = osc.step(P, _orc_preset(preset), [_oview(v) for v in views], imgs, 0, st, threads=1)
    assert np.allclose(losses, o["losses"], rtol=1e-9, atol=1e-15)
    _check_grad(R.getLastdLoss_dS(), o["grad"] * 3)          # before the batch division
    adam = R.get(dr.GET_ADAM)
    assert np.abs(adam[:P.size] - st[:P.size]).max() <= REL * np.abs(st[:P.size]).max()
    assert np.abs(adam[P.size:] - st[P.size:]).max() <= 3 * REL * np.abs(st[P.size:]).max()
    got = R.get(dr.GET_PARAMS)
    # the first Adam step moves each parameter by lr * g / (|g| + eps): equal where |g| is above noise
    big = np.abs(o["grad"]) > 1e-4 * np.abs(o["grad"]).max()
    assert big.sum() > 100
    assert np.abs(got - P)[big].max() <= 1e-3 * preset.opt_lr
    assert np.abs(got - P).max() <= 2.01 * preset.opt_lr
    R.close()


def test_reconstruction_lowers_the_loss():
    preset = dr.default_preset(border_spp=64, seed=2, opt_lr=1e-2, accumulate_batch=1)
    hdr, nodes, values, target, init, views = _problem(n_views=4, w=64, h=64)
    R = dr.MultiRendererDR()
    R.SetScene(hdr, nodes, values, target)
    imgs = _targets(R, views, target, preset)
    R.SetReference(imgs, [v[2] for v in views], [v[3] for v in views])
    sbs = [hdr, nodes, values, init.copy()]
    R.SetPreset(preset)
    R.set_params(init)
    first = R.step(0).mean()
    last = R.OptimizeFixedStructure(preset, sbs, 80, first_iter=1).mean()
    assert last < 0.7 * first, (first, last)
    assert not np.array_equal(sbs[3], init)
    R.close()


def test_host_rejects_bad_input():
    hdr, nodes, values, target, init, views = _problem(bc=3, bs=2)
    R = dr.MultiRendererDR()
    bad = nodes.copy()
    bad[0, 2] = values.size          # data offset past the end
    with pytest.raises(lrt.LrtError) as e:
        R.SetScene(hdr, bad, values, target)
    assert e.value.status == 6
    vals = values.copy()
    vals[0] = target.size + 5        # distance index past the parameters
    with pytest.raises(lrt.LrtError) as e:
        R.SetScene(hdr, nodes, vals, target)
    assert e.value.status == 6
    dx = lrt.SbsHeader(hdr.brick_size, hdr.brick_pad, hdr.bytes_per_value, lrt.SBS_LAYOUT_DX)
    with pytest.raises(lrt.LrtError) as e:
        R.SetScene(dx, nodes, values, target)
    assert e.value.status == 4
    with pytest.raises(lrt.LrtError):
        R.SetPreset(dr.default_preset(spp=65))
    with pytest.raises(lrt.LrtError) as e:
        R.render_grad(0)                 # no scene / reference yet
    assert e.value.status == 7
    R.close()


@pytest.mark.parametrize("flags,render_mode", [(8, dr.RENDER_LAMBERT), (1 | 2 | 4, dr.RENDER_LAMBERT), (8, dr.RENDER_MASK),
                                               (16, dr.RENDER_LINEAR_DEPTH)])
@pytest.mark.parametrize("layout_in", [True, False])
def test_query_rays_match_oracle(flags, render_mode, layout_in):
    """Per-ray RayQuery_NearestHitWithGrad: the hit and the border relaxation
    point (t, sdf, colour, normal, indices, dSDF/dtheta) bit for bit, on eye rays
    of three views and rays from random points, with the exact empty-voxel skips
    active on the GPU (the oracle walks every voxel)."""
    hdr, nodes, values, target, init, views = _problem(n_views=3, w=96, h=96, layout_in=layout_in)
    rng = np.random.default_rng(9)
    params = target.copy()
    nd = 25 ** 3
    params[:nd] += rng.normal(0, 0.004, nd).astype(np.float32)
    R = dr.MultiRendererDR()
    R.SetScene(hdr, nodes, values, params)
    R.SetPreset(dr.default_preset(render_mode=render_mode))
    P, D = [], []
    for (w, h, wv, pj) in views:
        p_, d_ = orc.eye_rays(w, h, lrt.inverse4x4(pj), lrt.inverse4x4(wv), np.arange(w * h, dtype=np.uint32),
                              0.37, 0.61)
        P.append(p_)
        D.append(d_)
    n = 6000
    rp = np.zeros((n, 4), np.float32)
    rp[:, :3] = rng.uniform(-1.6, 1.6, (n, 3))
    rd = np.zeros((n, 4), np.float32)
    d = rng.normal(size=(n, 3))
    rd[:, :3] = d / np.linalg.norm(d, axis=1, keepdims=True)
    rd[:, 3] = 1e9
    P.append(rp)
    D.append(rd)
    P, D = np.concatenate(P), np.concatenate(D)
    got = R.query_rays(flags, P, D)
    osc = _oracle(hdr, nodes, values, params, R.bvh2(), need_normal=render_mode in (1, 4))
    o = osc.query(params, flags, P, D).view(np.uint32).reshape(len(P), -1)
    want = np.concatenate([o[:, [0, 1]], o[:, 4:7], o[:, 8:11], o[:, [14, 21]], o[:, 18:21], o[:, 22:25],
                           o[:, 28:36], o[:, 36:44]], 1)
    assert (want[:, 1] != 0xFFFFFFFF).sum() > 3000
    if flags & 8:
        assert (want[:, 9].view(np.float32) < 1e-3).sum() > 50
    bad = np.nonzero((got != want).any(1))[0]
    assert bad.size == 0, (bad.size, bad[:5], got[bad[:2]], want[bad[:2]])
    R.close()
