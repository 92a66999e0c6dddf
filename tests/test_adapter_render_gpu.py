"""GPU: the engine driven as the reference-side binding drives it
(litert_gb300/ref_side/lrt_bvhrt_gpu.h: AddGeom_SdfSBS, AddInstance, CommitScene,
SetPreset, setSeed, the reference's BVH2 with its first-hit walk, one batched
RenderFloat) reproduces the reference's own MultiRenderer::RenderFloat
(CastRayFloatSingle over BVHRT::RayQuery_NearestHit, compiled in place and
recorded in tests/golden/ref_dr_glue.npz) bit for bit: regular and
RAY_GEN_MODE_RANDOM sub-pixel offsets, 1 to 9 samples per pixel."""
import os

import numpy as np
import pytest

import _dr_glue_cases as cases
from litert_gb300 import lrt

pytestmark = pytest.mark.gpu

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_dr_glue.npz"))


@pytest.mark.parametrize("i", range(len(cases.FWD_CASES)))
def test_render_float_equals_reference(i):
    rm, spp, rg, seed = cases.FWD_CASES[i]
    h, n, v, pairs, view = cases.fwd_inputs()
    s = lrt.Scene(0)
    try:
        s.add_instance(s.add_sbs(h, n, v))
        s.commit_scene()
        s.set_tuning("first_hit", 1)
        s.set_bvh2(pairs)
        s.set_seed(seed)
        s.set_preset(render_mode=rm, sdf_node_intersect=lrt.INTERSECT_NEWTON, spp=spp, ray_gen_mode=rg)
        col = s.render_host([view], rgba=True)["rgba"]
    finally:
        s.close()
    w, hh = view[0], view[1]
    assert cases.digest(col.reshape(hh, w, 4)) == str(GOLD[f"fwd{i}_digest"])
