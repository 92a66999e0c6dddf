"""Generate tests/golden/ref_dr_glue.npz from the reference's own
differentiable renderer and scene builders, compiled in place.

Runs where the reference tree is present: builds oracle/_ref/libref_dr.so
(oracle/build_ref.py: diff_render/MultiRendererDR.cpp, DR_common.cpp,
Renderer/eye_ray.cpp, utils/sparse_octree_builder.cpp, BVH2Common.cpp and
BVH2DR.cpp with oracle/ref_driver_dr.cpp) and records
  * create_sdf_SBS / create_sdf_SVS outputs (nodes, values) on the oracle's
    analytic SDFs,
  * create_grid_sbs outputs (indexed layout with the 27-neighbour table),
  * MultiRenderer::RenderFloat (SHA-256 digests of the colours) with the
    regular and RAY_GEN_MODE_RANDOM sub-pixel offsets,
  * MultiRendererDR::OptimizeFixedStructure on the cases of
    tests/_dr_glue_cases.py (one thread, setSeed): parameters after the last
    Adam step, the last gradient and the last images -- as arrays for two
    cases, as SHA-256 digests of the exact bytes for the rest.
tests/test_dr_glue_pin_cpu.py checks the oracle (and through it the engine)
against these outputs bit for bit.

    python tests/golden/make_golden_dr_glue.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

import _dr_glue_cases as cases  # noqa: E402
from oracle import ref_dr  # noqa: E402

OUT = os.path.join(HERE, "ref_dr_glue.npz")


def main():
    out = {}
    for i, (name, depth, bs, pad, bpv) in enumerate(cases.SBS_CASES):
        sp, bx, k = cases.sdf(name)
        h, n, v = ref_dr.build_sbs(sp, bx, k, depth, bs, pad, bpv)
        out[f"sbs{i}_hdr"] = np.array([h.brick_size, h.brick_pad, h.bytes_per_value, h.aux_data], np.uint32)
        out[f"sbs{i}_nodes"], out[f"sbs{i}_values"] = n, v
    for i, (name, depth) in enumerate(cases.SVS_CASES):
        sp, bx, k = cases.sdf(name)
        out[f"svs{i}_nodes"] = ref_dr.build_svs(sp, bx, k, depth)
    for i, (bc, bs, c, r, grad) in enumerate(cases.GRID_CASES):
        h, n, v, f = ref_dr.grid_sbs(bc, bs, c, r, grad)
        out[f"grid{i}_hdr"] = np.array([h.brick_size, h.brick_pad, h.bytes_per_value, h.aux_data], np.uint32)
        out[f"grid{i}_nodes"], out[f"grid{i}_values"], out[f"grid{i}_params"] = n, v, f
    h, n, v, pairs, view = cases.fwd_inputs()
    for i, (rm, spp, rg, seed) in enumerate(cases.FWD_CASES):
        out[f"fwd{i}_digest"] = np.array(cases.digest(ref_dr.render_float(h, n, v, pairs, view, rm, 2, spp, rg, seed)))
    target, init, pairs, views = cases.dr_inputs()
    ih, inn, iv, ip = init
    for c in cases.DR_CASES:
        imgs = cases.target_images(target, views, c["render_mode"])
        st = ref_dr.settings(**{k: v for k, v in c.items() if k != "name"}, image_batch_size=len(views),
                             lr=cases.DR_LR)
        p, g, im = ref_dr.optimize(ih, inn, iv, ip, pairs, imgs, [v[2] for v in views], [v[3] for v in views], st,
                                   cases.DR_SEED)
        out[f"dr_{c['name']}_digest"] = np.array(cases.digest(p, g, im))
        if c["name"] in cases.FULL_ARRAYS:
            out[f"dr_{c['name']}_params"], out[f"dr_{c['name']}_grad"], out[f"dr_{c['name']}_images"] = p, g, im
    np.savez_compressed(OUT, **out)
    print(OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
