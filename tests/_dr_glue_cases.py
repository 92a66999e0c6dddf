"""Inputs shared by tests/golden/make_golden_dr_glue.py and
tests/test_dr_glue_pin_cpu.py: the scenes, views, reference images and settings
on which the reference's MultiRendererDR::OptimizeFixedStructure, create_grid_sbs
and SDF -> SBS / SVS builders (compiled in place) recorded their outputs.
Everything here is rebuilt from code (the oracle's grids and SDF, the engine's
host BVH builder), so the fixture holds only the reference's outputs."""
import hashlib

import numpy as np

from litert_gb300 import lrt, scenes
from oracle import oracle as orc
from oracle import oracle_dr as od

# SDF -> SBS (depth, brick size, pad, bytes per value) and SDF -> SVS (depth)
SBS_CASES = [("sphere", 3, 4, 0, 4), ("union", 3, 4, 0, 4), ("union", 3, 2, 1, 2), ("sphere", 4, 8, 0, 1)]
SVS_CASES = [("sphere", 5), ("union", 4)]
# create_grid_sbs: (brick count, brick size, centre, radius, gradient colours)
GRID_CASES = [(4, 4, (0.0, 0.0, 0.0), 0.5, False), (3, 2, (0.0, -0.15, 0.0), 0.7, True)]
# OptimizeFixedStructure: reference-driver settings and iterations; two views of 32^2
DR_CASES = [
    dict(name="lambert_3iters", render_mode=1, reconstruction_flags=3, border_spp=32, iterations=3),
    dict(name="diffuse_colour", render_mode=0, reconstruction_flags=1, border_spp=0, iterations=1),
    dict(name="normal_geometry", render_mode=4, reconstruction_flags=2, border_spp=64, iterations=1),
    dict(name="regularisation", render_mode=1, reconstruction_flags=3, border_spp=16, iterations=2, reg_function=1),
    dict(name="redistancing", render_mode=1, reconstruction_flags=3, border_spp=16, iterations=2, redistancing_enable=1),
    dict(name="raycasting_mask", render_mode=1, reconstruction_flags=3, border_spp=16, iterations=3, raycasting_mask=1),
    dict(name="spp4", render_mode=1, reconstruction_flags=3, border_spp=16, iterations=1, spp=4),
    dict(name="mae", render_mode=1, reconstruction_flags=3, border_spp=16, iterations=1, loss_function=1),
    dict(name="depth_input", render_mode=3, reconstruction_flags=2, border_spp=16, iterations=1, input_type=1),
]
# MultiRenderer::RenderFloat on the union SBS (depth 4, 4-voxel bricks), one 64x72
# view: (render mode, spp, ray_gen_mode, seed)
FWD_CASES = [(8, 1, 0, 0), (8, 4, 1, 12345), (2, 4, 1, 7), (0, 9, 0, 0)]
DR_SEED = 9
DR_LR = 3e-3
DR_SIZE = 32
FULL_ARRAYS = ("lambert_3iters", "normal_geometry")   # cases stored as arrays, the rest as digests


def sdf(name):
    p = scenes.SPHERE_SDF if name == "sphere" else scenes.union_params()
    return p.get("spheres"), p.get("boxes"), p.get("k", 0.0)


def dr_inputs():
    """(target-grid scene, initial grid, pairs of the initial grid, views)."""
    up = scenes.union_params()
    target = od.grid_sbs(5, 4, spheres=up["spheres"], boxes=up["boxes"], k=up["k"], color=[0.8, 0.3, 0.2])
    init = od.grid_sbs(5, 4, spheres=np.array([[0, 0, 0, 0.55]], np.float32), color=[1, 0, 0])
    pairs = lrt.build_bvh2(orc.node_boxes(init[1]), 1)[0]
    views = [(DR_SIZE, DR_SIZE, lrt.look_at(e, [0, 0, 0], [0, 1, 0]), lrt.perspective(45.0, 1.0, 0.01, 100.0))
             for e in ([0.8, 1.0, 2.5], [-2.0, 0.5, 1.5])]
    return target, init, pairs, views


def target_images(target, views, render_mode):
    th, tn, tv, tp = target
    tsc = od.DrScene(th, tn, tv, tp.size, pairs=lrt.build_bvh2(orc.node_boxes(tn), 1)[0])
    pre = od.make_preset(render_mode=render_mode, reconstruction=0, border_spp=0, seed=DR_SEED)
    return [tsc.render(tp, pre, od.make_view(w, h, wv, pj, lrt.inverse4x4), np.zeros((w * h, 4), np.float32))
            ["image"].reshape(h, w, 4) for w, h, wv, pj in views]


def oracle_optimize(case, init, pairs, views, images):
    """The oracle's OptimizeFixedStructure restatement, one thread: (params, grad, images)."""
    ih, inn, iv, ip = init
    sc = od.DrScene(ih, inn, iv, ip.size, pairs=pairs)
    pre = od.make_preset(render_mode=case["render_mode"], reconstruction=case["reconstruction_flags"],
                         border_spp=case["border_spp"], seed=DR_SEED, lr=DR_LR, spp=case.get("spp", 1),
                         loss=case.get("loss_function", 0), input_type=case.get("input_type", 0),
                         reg_function=case.get("reg_function", 0),
                         redistancing_enable=case.get("redistancing_enable", 0),
                         raycasting_mask=case.get("raycasting_mask", 0))
    params = ip.copy()
    state = np.zeros(2 * ip.size, np.float32)
    masks = [np.ones(w * h, np.uint8) for w, h, _, _ in views] if case.get("raycasting_mask") else None
    ovs = [od.make_view(w, h, wv, pj, lrt.inverse4x4) for w, h, wv, pj in views]
    out = None
    for it in range(case["iterations"]):
        out = sc.step(params, pre, ovs, images, it, state, threads=1, masks=masks)
    return params, out["grad"], out["images"].reshape(len(views), views[0][1], views[0][0], 4)


def digest(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def fwd_inputs():
    h, n, v = lrt.sbs_from_sdf(lrt.Sdf(**scenes.union_params()), 4, 4)
    pairs = lrt.build_bvh2(orc.node_boxes(n), 1)[0]
    return h, n, v, pairs, scenes.union_views(n_views=1, lo=64, hi=72)[0]


def oracle_render_float(h, n, v, pairs, view, rm, spp, rg, seed):
    """The oracle in the reference's first-hit mode on the same BVH2."""
    w, hh, wv, pj = view
    osc = orc.Scene("sbs", sbs=(orc.SbsHeader(h.brick_size, h.brick_pad, h.bytes_per_value, h.aux_data), n, v),
                    pairs=(pairs, None, None), intersect=2, render_mode=rm, closest_hit=False, spp=spp,
                    ray_gen_mode=rg, seed=seed)
    _, col, _ = osc.render(w, hh, lrt.inverse4x4(pj), lrt.inverse4x4(wv), hits=False, rgba=True)
    return col.reshape(hh, w, 4)
