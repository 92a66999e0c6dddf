"""GPU: the engine's differentiable renderer against outputs of the reference's
own MultiRendererDR::OptimizeFixedStructure, compiled in place
(tests/golden/ref_dr_glue.npz, tests/golden/make_golden_dr_glue.py).

Same indexed SBS, BVH2, views, reference images, seed and settings as the
recorded reference run.  After the first iteration the rendered images are
bit-identical to the reference's; the last gradient handed to Adam -- interior
term plus the random border integral -- is within 1e-3 of the reference's in
norm (the engine sums per-pixel partial derivatives with atomics, so the float
additions happen in another order); the parameters after the last Adam step are
within 1e-3 of the reference's step.  Over several iterations the summation
order feeds back through the parameters, so later images are compared within
the same tolerance."""
import os

import numpy as np
import pytest

import _dr_glue_cases as cases
from litert_gb300 import dr, lrt

pytestmark = pytest.mark.gpu

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_dr_glue.npz"))


@pytest.mark.parametrize("name", cases.FULL_ARRAYS)
def test_engine_optimize_matches_reference_run(name):
    case = next(c for c in cases.DR_CASES if c["name"] == name)
    target, init, pairs, views = cases.dr_inputs()
    imgs = cases.target_images(target, views, case["render_mode"])
    hdr, nodes, values, params = init
    R = dr.MultiRendererDR()
    try:
        R.SetReference(imgs, [v[2] for v in views], [v[3] for v in views])
        R.SetPreset(dr.default_preset(render_mode=case["render_mode"],
                                      reconstruction_flags=case["reconstruction_flags"],
                                      border_spp=case["border_spp"], seed=cases.DR_SEED, opt_lr=cases.DR_LR, spp=1))
        R.SetScene(lrt.SbsHeader(hdr.brick_size, hdr.brick_pad, hdr.bytes_per_value, hdr.aux_data), nodes, values,
                   params.copy(), pairs=pairs)
        assert np.array_equal(R.bvh2(), np.ascontiguousarray(pairs).view(np.uint8).reshape(-1))
        for it in range(case["iterations"]):
            R.step(it)
        g = R.getLastdLoss_dS() / np.float32(len(views))   # LRT_DR_GRAD is taken before the batch division
        p = R.get(dr.GET_PARAMS)
        got = np.stack([R.getLastImage(k) for k in range(len(views))])
    finally:
        R.close()
    G, P, I = GOLD[f"dr_{name}_grad"], GOLD[f"dr_{name}_params"], GOLD[f"dr_{name}_images"]
    assert np.linalg.norm(G) > 0
    assert np.linalg.norm(g - G) <= 1e-3 * np.linalg.norm(G), np.linalg.norm(g - G) / np.linalg.norm(G)
    assert np.linalg.norm(p - P) <= 1e-3 * np.linalg.norm(P - params)
    if case["iterations"] == 1:
        assert np.array_equal(got.view(np.uint32), I.view(np.uint32))
    else:
        assert np.abs(got - I).max() <= 1e-2 and np.mean(np.abs(got - I)) <= 1e-4
