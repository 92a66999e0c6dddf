"""GPU: Regularization and Redistance in the optimisation step against the oracle.
With lr 0 Adam leaves the parameters alone, so after a step with redistancing the
GPU's parameters are the redistanced grid, equal to the oracle's bit for bit (a
deterministic Jacobi sweep); the step's gradient with regularisation on equals
the oracle's within the gradient bar (1e-3; atomics sum in another order)."""
import numpy as np
import pytest

from litert_gb300 import dr, lrt, scenes
from oracle import oracle as orc
from oracle import oracle_dr as od

pytestmark = pytest.mark.gpu


def _setup(**kw):
    up = scenes.union_params()
    sdf_t = lrt.Sdf(up["spheres"], up["boxes"], up["k"])
    hdr, nodes, values, target = dr.grid_sbs(6, 4, sdf_t, None)
    _, _, _, init = dr.grid_sbs(6, 4, lrt.Sdf(spheres=np.array([[0, 0, 0, 0.55]], np.float32)), [0.8, 0.3, 0.2])
    pj = lrt.perspective(45.0, 1.0, 0.01, 100.0)
    views = [(48, 48, lrt.look_at([2.6 * np.sin(a), 1.0, 2.6 * np.cos(a)], [0, 0, 0], [0, 1, 0]), pj)
             for a in (0.3, 2.0)]
    R = dr.MultiRendererDR()
    R.SetScene(hdr, nodes, values, target)
    R.SetReference([np.zeros((48, 48, 4), np.float32)] * 2, [v[2] for v in views], [v[3] for v in views])
    R.SetPreset(dr.default_preset(reconstruction_flags=0, border_spp=0))
    imgs = []
    for i in range(2):
        R.render_grad(i)
        imgs.append(R.getLastImage(i).copy())
    R.set_params(init)
    R.SetReference(imgs, [v[2] for v in views], [v[3] for v in views])
    preset = dr.default_preset(border_spp=16, seed=3, accumulate_batch=1, **kw)
    R.SetPreset(preset)
    osc = od.DrScene(orc.SbsHeader(hdr.brick_size, hdr.brick_pad, hdr.bytes_per_value, hdr.aux_data), nodes, values,
                     init.size, pairs=R.bvh2())
    lights = [(preset.lights[i].type, np.array(preset.lights[i].dir[:], np.float32),
               np.array(preset.lights[i].color[:], np.float32)) for i in range(preset.n_lights)]
    op = od.make_preset(render_mode=preset.render_mode, reconstruction=preset.reconstruction_flags,
                        border_spp=preset.border_spp, seed=preset.seed, lights=lights, lr=preset.opt_lr,
                        accumulate_batch=1, reg_function=preset.reg_function, reg_lambda=preset.reg_lambda,
                        reg_power=preset.reg_power, redistancing_enable=preset.redistancing_enable,
                        redistancing_interval=preset.redistancing_interval)
    oviews = [od.make_view(v[0], v[1], v[2], v[3], lrt.inverse4x4) for v in views]
    return R, osc, init, op, oviews, imgs


def test_regularization_in_the_step():
    R, osc, init, op, oviews, imgs = _setup(reg_function=1, reg_lambda=20.0, reg_power=2.0, opt_lr=0.0)
    R.step(0)
    g = R.get(dr.GET_GRAD)
    params = init.copy()
    state = np.zeros(2 * params.size, np.float32)
    o = osc.step(params, op, oviews, imgs, 0, state, threads=1)
    reg = osc.regularize(init, op) / 2   # the regularisation part of the (batch-divided) gradient
    assert np.linalg.norm(reg) > 0.1 * np.linalg.norm(o["grad"])
    want = o["grad"] * 2          # the engine's buffer holds the batch sum, before the division
    nrm = np.linalg.norm(want)
    assert np.linalg.norm(g - want) <= 1e-3 * nrm
    R.close()


def test_redistancing_in_the_step():
    R, osc, init, op, oviews, imgs = _setup(redistancing_enable=1, redistancing_interval=1, opt_lr=0.0)
    R.step(0)
    got = R.get(dr.GET_PARAMS)
    params = init.copy()
    state = np.zeros(2 * params.size, np.float32)
    osc.step(params, op, oviews, imgs, 0, state, threads=1)
    assert not np.array_equal(params, init)
    assert np.array_equal(got.view(np.uint32), params.view(np.uint32))
    R.close()
