"""GPU parity of the SBS primary-ray kernel against the CPU oracle.

Bar: bit-exact hit records (t, primId, octahedral normal) and hit mask on every
pixel, because both sides evaluate the reference's FP32 expressions in the same
order without contraction.  The ANALYTIC finder calls acosf/cosf/powf whose
last-ulp results differ between CUDA and glibc; there the bar is the
forward tolerance of the path: identical mask except <0.01% of pixels, |dt| <= 1e-4 of
the scene extent (2), normals within 1e-3.
"""
import numpy as np
import pytest

from litert_gb300 import lrt, scenes
from oracle import oracle as orc

from _util import compare_hits16, gpu_scene_sbs, orc_header, oracle_render, records_equal, sbs_scene

pytestmark = pytest.mark.gpu
EXTENT = 2.0


def _run(params, depth, bs, view, intersect=lrt.INTERSECT_NEWTON, render_mode=lrt.RENDER_MODE_NORMAL, pad=0, bpv=4, variant=1,
         representation_mode=1):
    h, n, v = sbs_scene(params, depth, bs, pad, bpv)
    g = gpu_scene_sbs(h, n, v, variant=variant, render_mode=render_mode, sdf_node_intersect=intersect,
                      representation_mode=representation_mode)
    out = g.render_host([view], hits=True, rgba=True, rgba8=True)
    osc = orc.Scene("sbs", sbs=(orc_header(h), n, v), intersect=intersect, render_mode=render_mode,
                    representation_mode=representation_mode)
    hits, col, cnt = oracle_render(osc, view)
    g.close()
    return out, hits, col


VARIANTS = [0, 1]   # one ray per lane / warp packet with shared-memory brick staging


@pytest.mark.parametrize("variant", VARIANTS)
@pytest.mark.parametrize("intersect", [lrt.INTERSECT_NEWTON, lrt.INTERSECT_ST, lrt.INTERSECT_BBOX, lrt.INTERSECT_IT])
def test_sphere_config_bit_exact(intersect, variant):
    out, hits, col = _run(scenes.SPHERE_SDF, 4, 4, scenes.sphere_view(), intersect=intersect, variant=variant)
    r = compare_hits16(out["hits"], hits)
    assert r["hits"] > 5000, r
    assert r["mask"] == 0 and r["t"] == 0 and r["prim"] == 0 and r["nx"] == 0 and r["ny"] == 0, r
    assert np.array_equal(out["rgba"].view(np.uint32), col.view(np.uint32))


def test_sphere_analytic_within_tolerance():
    out, hits, col = _run(scenes.SPHERE_SDF, 4, 4, scenes.sphere_view(), intersect=lrt.INTERSECT_ANALYTIC)
    g, o = out["hits"], hits
    mg, mo = g["primId"] != lrt.MISS, o["primId"] != lrt.MISS
    assert (mg != mo).sum() <= 1e-4 * g.size
    both = mg & mo
    assert np.abs(g["t"][both] - o["t"][both]).max() <= 1e-4 * EXTENT
    assert np.abs(g["nx"][both] - o["coords"][both, 2]).max() <= 1e-3
    assert np.abs(g["ny"][both] - o["coords"][both, 3]).max() <= 1e-3


def test_sphere_literal_depth6():
    """Literal reading of the config (depth 6, 4-voxel bricks: 256^3)."""
    out, hits, _ = _run(scenes.SPHERE_SDF, 6, 4, scenes.sphere_view())
    r = compare_hits16(out["hits"], hits)
    assert r["mask"] == 0 and r["t"] == 0 and r["prim"] == 0 and r["nx"] == 0, r


@pytest.mark.parametrize("variant", VARIANTS)
@pytest.mark.parametrize("bpv,pad,bs", [(1, 0, 4), (2, 1, 2), (4, 1, 8), (1, 0, 1), (2, 0, 16)])
def test_layout_variants(bpv, pad, bs, variant):
    out, hits, _ = _run(scenes.SPHERE_SDF, 4, bs, scenes.sphere_view(128, 96), pad=pad, bpv=bpv, variant=variant)
    r = compare_hits16(out["hits"], hits)
    assert r["mask"] == 0 and r["t"] == 0 and r["prim"] == 0 and r["nx"] == 0 and r["ny"] == 0, r


@pytest.mark.parametrize("mode", [lrt.RENDER_MODE_MASK, lrt.RENDER_MODE_LAMBERT_NO_TEX, lrt.RENDER_MODE_DEPTH,
                                  lrt.RENDER_MODE_LINEAR_DEPTH, lrt.RENDER_MODE_INVERSE_LINEAR_DEPTH])
@pytest.mark.parametrize("variant", VARIANTS)
def test_render_modes(mode, variant):
    out, hits, col = _run(scenes.SPHERE_SDF, 4, 4, scenes.sphere_view(96, 64), render_mode=mode, variant=variant)
    assert np.array_equal(out["rgba"].view(np.uint32), col.view(np.uint32))
    # RGBA8 packing of MultiRenderer::CastRaySingle (Renderer/eye_ray.cpp:111-115)
    c = np.clip(col, 0, 1)
    q = (255 * c).astype(np.uint32)
    ref8 = q[:, 0] | (q[:, 1] << 8) | (q[:, 2] << 16) | (q[:, 3] << 24)
    assert np.array_equal(out["rgba8"], ref8)


def test_surface_representation_mode():
    out, hits, _ = _run(scenes.SPHERE_SDF, 4, 4, scenes.sphere_view(128, 128), representation_mode=0)
    r = compare_hits16(out["hits"], hits)
    assert r["mask"] == 0 and r["t"] == 0 and r["nx"] == 0, r


@pytest.mark.parametrize("variant,stage", [(0, 0), (1, 0), (1, 1)])
def test_union_scene_multi_view(variant, stage):
    """Config-3 scene at reduced depth, three views of different sizes in one launch;
    the packet kernel with and without shared-memory brick staging."""
    p = scenes.union_params()
    h, n, v = sbs_scene(p, 5, 4)
    views = scenes.union_views(n_views=3, lo=96, hi=200)
    g = gpu_scene_sbs(h, n, v, variant=variant, render_mode=lrt.RENDER_MODE_NORMAL,
                      sdf_node_intersect=lrt.INTERSECT_NEWTON)
    g.set_tuning("stage", stage)
    out = g.render_host(views, hits=True)
    osc = orc.Scene("sbs", sbs=(orc_header(h), n, v), intersect=lrt.INTERSECT_NEWTON, render_mode=lrt.RENDER_MODE_NORMAL)
    off = 0
    for view in views:
        w, hh = view[0], view[1]
        hits, _, _ = oracle_render(osc, view)
        r = compare_hits16(out["hits"][off:off + w * hh], hits)
        assert r["hits"] > 0 and r["mask"] == 0 and r["t"] == 0 and r["prim"] == 0 and r["nx"] == 0, r
        off += w * hh
    g.close()


def test_query_rays_random_and_anyhit():
    h, n, v = sbs_scene(scenes.SPHERE_SDF, 4, 4)
    g = gpu_scene_sbs(h, n, v, render_mode=lrt.RENDER_MODE_NORMAL, sdf_node_intersect=lrt.INTERSECT_NEWTON)
    rng = np.random.default_rng(0)
    N = 20000
    pos = np.zeros((N, 4), np.float32)
    pos[:, :3] = rng.uniform(-2, 2, (N, 3))
    pos[:, 3] = rng.choice([0.0, 0.5], N)
    d = rng.normal(size=(N, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    dirs = np.zeros((N, 4), np.float32)
    dirs[:, :3] = d
    dirs[:, 3] = 1e9
    gh = g.query_rays(pos, dirs)
    osc = orc.Scene("sbs", sbs=(orc_header(h), n, v), intersect=lrt.INTERSECT_NEWTON, render_mode=lrt.RENDER_MODE_NORMAL)
    oh = osc.query_rays(pos, dirs)
    assert records_equal(gh, oh)
    # any-hit (tFar < 0): hit/miss agrees with the nearest-hit query
    dirs[:, 3] = -1e9
    ga = g.query_rays(pos, dirs)
    assert np.array_equal(ga["primId"] != lrt.MISS, oh["primId"] != lrt.MISS)
    g.close()


def test_error_paths():
    s = lrt.Scene(0)
    with pytest.raises(lrt.LrtError):
        s.render_host([scenes.sphere_view(8, 8)])          # not committed
    with pytest.raises(lrt.LrtError):
        s.commit_scene()                                     # no instance
    h, n, v = sbs_scene(scenes.SPHERE_SDF, 4, 4)
    bad = n.copy()
    bad[0, 2] = v.size                                       # data offset out of range
    with pytest.raises(lrt.LrtError):
        s.add_sbs(h, bad, v)
    s.close()
