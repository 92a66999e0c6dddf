"""GPU: MultiRendererDR::OptimizeGrid (diff_render/MultiRendererDR.cpp:228-276).

With learning rate 0 the optimisation leaves every stage's parameters alone, so
the final grid is the starting grid resampled stage after stage and must equal
the oracle's chain of resamples bit for bit (growing after every stage, or not
after the last).  With a learning rate the loss of the final stage falls below
the loss of the same schedule cut to one iteration per stage, with the host and
both device BVH builders alike."""
import numpy as np
import pytest

from litert_gb300 import dr, lrt, scenes
from oracle import oracle_dr as od

pytestmark = pytest.mark.gpu

S = 40


def _renderer(bvh_builder=0):
    up = scenes.union_params()
    hdr, nodes, values, target = dr.grid_sbs(6, 4, lrt.Sdf(up["spheres"], up["boxes"], up["k"]), None)
    pj = lrt.perspective(45.0, 1.0, 0.01, 100.0)
    wvs = [lrt.look_at([2.6 * np.sin(a), 1.0, 2.6 * np.cos(a)], [0, 0, 0], [0, 1, 0]) for a in (0.3, 2.0, 4.0)]
    R = dr.MultiRendererDR()
    R.set_tuning("bvh_builder", bvh_builder)
    R.SetScene(hdr, nodes, values, target)
    R.SetReference([np.zeros((S, S, 4), np.float32)] * 3, wvs, [pj] * 3)
    R.SetPreset(dr.default_preset(reconstruction_flags=0, border_spp=0))
    imgs = []
    for i in range(3):
        R.render_grad(i)
        imgs.append(R.getLastImage(i).copy())
    R.SetReference(imgs, wvs, [pj] * 3)
    return R


@pytest.mark.parametrize("no_last_step_resize", [False, True])
def test_optimize_grid_zero_lr_is_the_resample_chain(no_last_step_resize):
    R = _renderer()
    presets = [dr.default_preset(opt_lr=0.0, border_spp=16, seed=s) for s in (1, 2)]
    grid, _ = R.OptimizeGrid(4, no_last_step_resize, presets, [2, 2])
    R.close()
    p = od.grid_resample(4, 1)
    p = od.grid_resample(4, 2, p, 1)
    p = od.grid_resample(4, 2 if no_last_step_resize else 4, p, 2)
    assert grid[0].brick_size == (2 if no_last_step_resize else 4)
    assert np.array_equal(grid[3].view(np.uint32), p.view(np.uint32))


@pytest.mark.parametrize("bvh_builder", [0, 1, 2])
def test_optimize_grid_reduces_the_loss(bvh_builder):
    presets = [dr.default_preset(opt_lr=0.02, border_spp=16, seed=3, accumulate_batch=1),
               dr.default_preset(opt_lr=0.01, border_spp=16, seed=4, accumulate_batch=1)]
    R = _renderer(bvh_builder)
    _, short = R.OptimizeGrid(4, True, presets, [1, 1])
    R.close()
    R = _renderer(bvh_builder)
    grid, long = R.OptimizeGrid(4, True, presets, [30, 30])
    R.close()
    assert grid[0].brick_size == 2
    assert np.all(np.isfinite(long)) and long.mean() < 0.8 * short.mean()


def test_optimize_grid_per_stage_render_size():
    """Each stage renders the reference resampled to its own size (the reference's
    preset render_width/height): the context ends at the last stage's size and the
    loss still falls."""
    presets = [dr.default_preset(opt_lr=0.02, border_spp=16, seed=3, accumulate_batch=1),
               dr.default_preset(opt_lr=0.01, border_spp=16, seed=4, accumulate_batch=1)]
    sizes = [(24, 24), (32, 32)]
    R = _renderer()
    _, short = R.OptimizeGrid(4, True, presets, [1, 1], render_sizes=sizes)
    R.close()
    R = _renderer()
    grid, long = R.OptimizeGrid(4, True, presets, [30, 30], render_sizes=sizes)
    img = np.zeros((32 * 32, 4), np.float32)
    R._chk(dr._lib().lrt_dr_get(R._ctx, dr.GET_IMAGE, 0, lrt._ptr(img), img.nbytes))
    R.close()
    assert img[:, 3].max() > 0
    assert np.all(np.isfinite(long)) and long.mean() < 0.8 * short.mean()

