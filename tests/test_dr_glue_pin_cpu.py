"""CPU: the oracle's restatements of the differentiable renderer's glue and of
scene construction, pinned to the reference's own code compiled in place.

Fixture tests/golden/ref_dr_glue.npz (tests/golden/make_golden_dr_glue.py) holds
what the reference produced for the cases of tests/_dr_glue_cases.py:
  * create_sdf_SBS / create_sdf_SVS (utils/sdf_converter.cpp:118-181 over
    utils/sparse_octree_builder.cpp:72-444): the oracle's builders and the
    engine's host builders return the same nodes and values, bit for bit;
  * create_grid_sbs with the 27-neighbour table (diff_render/DR_common.cpp:47-146,
    utils/sparse_octree_builder.cpp:2761-2850): the oracle's and the engine's
    grids are bit-identical;
  * MultiRendererDR::OptimizeFixedStructure (diff_render/MultiRendererDR.cpp:278-576:
    RenderDR with CastRayWithGrad, the border-pixel search and the random border
    integral, Loss/LossGrad, getBaseGradientMult, Regularization, Redistance,
    the ray-casting mask and OptimizeStepAdam) over 1-3 iterations on two views:
    the oracle's parameters, last gradient and images are bit-identical.
  * MultiRenderer::RenderFloat with regular and random (RAY_GEN_MODE_RANDOM)
    sub-pixel offsets: the oracle's colours are bit-identical.
Where the reference tree is present the same comparisons also run live, plus
cases outside the fixture."""
import numpy as np
import pytest

import _dr_glue_cases as cases
from litert_gb300 import dr, lrt
from oracle import oracle as orc
from oracle import oracle_dr as od

GOLD = np.load(__import__("os").path.join(__import__("os").path.dirname(__file__), "golden", "ref_dr_glue.npz"))

live = pytest.mark.skipif(not __import__("oracle.ref_dr", fromlist=["x"]).available(),
                          reason="reference tree not present (pinned through the golden fixture instead)")


@pytest.mark.parametrize("i", range(len(cases.SBS_CASES)))
def test_sbs_builder_matches_reference(i):
    name, depth, bs, pad, bpv = cases.SBS_CASES[i]
    sp, bx, k = cases.sdf(name)
    hdr, nodes, values = orc.build_sbs(sp, bx, k, depth, bs, pad, bpv)
    assert np.array_equal([hdr.brick_size, hdr.brick_pad, hdr.bytes_per_value, hdr.aux_data], GOLD[f"sbs{i}_hdr"])
    assert np.array_equal(nodes, GOLD[f"sbs{i}_nodes"]) and np.array_equal(values, GOLD[f"sbs{i}_values"])
    eh, en, ev = lrt.sbs_from_sdf(lrt.Sdf(spheres=sp, boxes=bx, k=k), depth, bs, pad, bpv)
    assert np.array_equal(en, GOLD[f"sbs{i}_nodes"]) and np.array_equal(ev, GOLD[f"sbs{i}_values"])


@pytest.mark.parametrize("i", range(len(cases.SVS_CASES)))
def test_svs_builder_matches_reference(i):
    name, depth = cases.SVS_CASES[i]
    sp, bx, k = cases.sdf(name)
    assert np.array_equal(orc.build_svs(sp, bx, k, depth), GOLD[f"svs{i}_nodes"])
    assert np.array_equal(lrt.svs_from_sdf(lrt.Sdf(spheres=sp, boxes=bx, k=k), depth), GOLD[f"svs{i}_nodes"])


def test_grid_sbs_matches_reference():
    bc, bs, c, r, grad = cases.GRID_CASES[0]
    sph = np.array([[c[0], c[1], c[2], r]], np.float32)
    for h, n, v, f in (od.grid_sbs(bc, bs, spheres=sph, color=[1, 0, 0]),
                       dr.grid_sbs(bc, bs, lrt.Sdf(spheres=sph), [1, 0, 0])):
        assert np.array_equal([h.brick_size, h.brick_pad, h.bytes_per_value, h.aux_data], GOLD["grid0_hdr"])
        assert np.array_equal(n, GOLD["grid0_nodes"]) and np.array_equal(v, GOLD["grid0_values"])
        assert np.array_equal(f.view(np.uint32), GOLD["grid0_params"].view(np.uint32))
    # gradient colours: OptimizeGrid's starting grid (circle_sdf((0,-0.15,0), 0.7), gradient_color)
    bc, bs, c, r, grad = cases.GRID_CASES[1]
    start = od.grid_resample(bc, bs)
    assert np.array_equal(start.view(np.uint32), GOLD["grid1_params"].view(np.uint32))


@pytest.mark.parametrize("i", range(len(cases.FWD_CASES)))
def test_render_float_matches_reference(i):
    """MultiRenderer::RenderFloat -> CastRayFloatSingle (Renderer/eye_ray.cpp:118-142):
    the spp loop with the regular grid and with RAY_GEN_MODE_RANDOM's
    rand2(x, y, i + m_seed % 2) offsets, eye rays, the first-hit query and
    kernel_RayTrace's colour, bit for bit."""
    rm, spp, rg, seed = cases.FWD_CASES[i]
    col = cases.oracle_render_float(*cases.fwd_inputs(), rm, spp, rg, seed)
    assert (col[..., 0] > 0).sum() > 1000
    assert cases.digest(col) == str(GOLD[f"fwd{i}_digest"])


@pytest.mark.parametrize("case", cases.DR_CASES, ids=[c["name"] for c in cases.DR_CASES])
def test_optimize_fixed_structure_matches_reference(case):
    target, init, pairs, views = cases.dr_inputs()
    imgs = cases.target_images(target, views, case["render_mode"])
    p, g, im = cases.oracle_optimize(case, init, pairs, views, imgs)
    assert np.linalg.norm(g) > 0
    name = case["name"]
    if name in cases.FULL_ARRAYS:
        assert np.array_equal(p.view(np.uint32), GOLD[f"dr_{name}_params"].view(np.uint32))
        assert np.array_equal(g.view(np.uint32), GOLD[f"dr_{name}_grad"].view(np.uint32))
        assert np.array_equal(im.view(np.uint32), GOLD[f"dr_{name}_images"].view(np.uint32))
    assert cases.digest(p, g, im) == str(GOLD[f"dr_{name}_digest"])


@live
def test_live_builders_and_grid_match_reference():
    from oracle import ref_dr
    for name, depth, bs, pad, bpv in (("union", 4, 4, 0, 4), ("union", 4, 8, 1, 2), ("sphere", 5, 4, 0, 1)):
        sp, bx, k = cases.sdf(name)
        rh, rn, rv = ref_dr.build_sbs(sp, bx, k, depth, bs, pad, bpv)
        oh, on, ov = orc.build_sbs(sp, bx, k, depth, bs, pad, bpv)
        assert np.array_equal(rn, on) and np.array_equal(rv, ov)
    rs = ref_dr.build_svs(*cases.sdf("union"), 5)
    assert np.array_equal(rs, orc.build_svs(*cases.sdf("union"), 5))
    for bc, bs, r in ((6, 2, 0.55), (8, 1, 0.7), (3, 8, 0.5)):
        rh, rn, rv, rf = ref_dr.grid_sbs(bc, bs, (0, 0, 0), r, False)
        oh, on, ov, of = od.grid_sbs(bc, bs, spheres=np.array([[0, 0, 0, r]], np.float32), color=[1, 0, 0])
        assert np.array_equal(rn, on) and np.array_equal(rv, ov) and np.array_equal(rf.view(np.uint32),
                                                                                     of.view(np.uint32))


@live
def test_live_adam_matches_reference():
    from oracle import ref_dr
    rng = np.random.default_rng(1)
    n = 50000
    x0 = rng.normal(0, 0.5, n).astype(np.float32)
    xs, ss = [x0.copy(), x0.copy()], [np.zeros(2 * n, np.float32), np.zeros(2 * n, np.float32)]
    for it in range(4):
        g = (rng.normal(0, 1, n) * 10 ** rng.uniform(-6, 2, n)).astype(np.float32)
        ref_dr.adam(it, g, xs[0], ss[0], 3e-3)
        od.adam(it, g, xs[1], ss[1], 3e-3)
        assert np.array_equal(xs[0].view(np.uint32), xs[1].view(np.uint32))
        assert np.array_equal(ss[0].view(np.uint32), ss[1].view(np.uint32))


@live
@pytest.mark.parametrize("views_seed", [0, 1])
def test_live_optimize_matches_reference(views_seed):
    from oracle import ref_dr
    target, init, pairs, _ = cases.dr_inputs()
    rng = np.random.default_rng(views_seed)
    views = []
    for _ in range(3):
        e = rng.normal(size=3)
        e = 2.8 * e / np.linalg.norm(e)
        views.append((40, 24, lrt.look_at(e, [0, 0, 0], [0, 1, 0]), lrt.perspective(50.0, 40 / 24, 0.01, 100.0)))
    imgs = cases.target_images(target, views, 1)
    case = dict(render_mode=1, reconstruction_flags=3, border_spp=48, iterations=2)
    ih, inn, iv, ip = init
    st = ref_dr.settings(**case, image_batch_size=3, lr=cases.DR_LR)
    rp, rg, ri = ref_dr.optimize(ih, inn, iv, ip, pairs, imgs, [v[2] for v in views], [v[3] for v in views], st,
                                 cases.DR_SEED)
    p, g, im = cases.oracle_optimize(case, init, pairs, views, imgs)
    assert np.array_equal(p.view(np.uint32), rp.view(np.uint32))
    assert np.array_equal(g.view(np.uint32), rg.view(np.uint32))
    assert np.array_equal(im.view(np.uint32), ri.view(np.uint32))


@live
def test_live_render_float_matches_reference():
    from oracle import ref_dr
    h, n, v, pairs, _ = cases.fwd_inputs()
    view = __import__("litert_gb300.scenes", fromlist=["x"]).union_views(n_views=1, lo=40, hi=56, cam_seed=9)[0]
    for rm, spp, rg, seed in ((8, 4, 1, 99), (3, 16, 1, 4), (8, 4, 0, 0)):
        ref = ref_dr.render_float(h, n, v, pairs, view, rm, 2, spp, rg, seed)
        assert np.array_equal(ref.view(np.uint32), cases.oracle_render_float(h, n, v, pairs, view, rm, spp, rg,
                                                                              seed).view(np.uint32))
