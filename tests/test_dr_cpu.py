"""CPU: host side of the differentiable render.

create_grid_sbs + the neighbour table built by the engine's host code
(lrt_dr_grid_sbs) equal the oracle's restatement of
diff_render/DR_common.cpp:47-146 and utils/sparse_octree_builder.cpp:2761-2850
word for word, and the default preset carries getDefaultPresetDR's values.
"""
import numpy as np
import pytest

from litert_gb300 import dr, lrt, scenes
from oracle import oracle_dr as od


@pytest.mark.parametrize("bc,bs,color", [(4, 4, [1, 0, 0]), (3, 8, None), (5, 2, [0.2, 0.4, 0.6])])
def test_grid_sbs_matches_oracle(bc, bs, color):
    up = scenes.union_params()
    sdf = lrt.Sdf(up["spheres"], up["boxes"], up["k"])
    h1, n1, v1, p1 = dr.grid_sbs(bc, bs, sdf, color)
    h2, n2, v2, p2 = od.grid_sbs(bc, bs, spheres=up["spheres"], boxes=up["boxes"], k=up["k"], color=color)
    assert (h1.brick_size, h1.brick_pad, h1.bytes_per_value, h1.aux_data) == \
           (h2.brick_size, h2.brick_pad, h2.bytes_per_value, h2.aux_data)
    assert np.array_equal(n1, n2)
    assert np.array_equal(v1, v2)
    assert np.array_equal(p1.view(np.uint32), p2.view(np.uint32))


def test_sphere_grid_matches_oracle():
    sdf = lrt.Sdf(spheres=np.array([[0, 0, 0, 0.5]], np.float32))
    a = dr.grid_sbs(8, 4, sdf, [1, 0, 0])
    b = od.grid_sbs(8, 4, spheres=np.array([[0, 0, 0, 0.5]], np.float32), color=[1, 0, 0])
    assert all(np.array_equal(np.asarray(x).view(np.uint32), np.asarray(y).view(np.uint32)) for x, y in zip(a[1:], b[1:]))


def test_default_preset():
    p = dr.default_preset()
    assert (p.spp, p.border_spp, p.loss_function, p.input_type) == (1, 256, 0, 0)
    assert abs(p.border_relax_eps - 1e-3) < 1e-9 and abs(p.opt_lr - 0.01) < 1e-9
    assert abs(p.opt_beta_1 - 0.9) < 1e-7 and abs(p.opt_beta_2 - 0.999) < 1e-7 and abs(p.opt_eps - 1e-8) < 1e-12
    assert p.n_lights == 2 and p.lights[0].type == 0 and p.lights[1].type == 2
    d = np.array(p.lights[0].dir[:], np.float32)
    want = od.default_lights()[0][1]
    assert np.array_equal(d, want)
