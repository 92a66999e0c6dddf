"""GPU: the render kernels compiled with floating-point contraction ("fma" tuning).

These kernels contract a * b + c into one FMA, so they are not bit-identical to
the reference's x86-64 build; the bar is the forward parity tolerance for the
path: identical hit mask except below 0.01 % of pixels, depth within 1e-4 of the
scene extent on every pixel both sides hit, normals within 1e-3 except below
0.01 % of pixels (grazing and crease pixels, where the hit falls into the
neighbouring voxel and the trilinear gradient jumps).  Checked against the
oracle at the oracle's sizes and against the bit-exact kernel (itself checked
bit for bit against the oracle) on the full 1024^3 union scene."""
import numpy as np
import pytest

from litert_gb300 import lrt, scenes
from oracle import oracle as orc

from _util import gpu_scene_sbs, orc_header, oracle_render, sbs_scene

pytestmark = pytest.mark.gpu
EXTENT = 2.0
FRAC = 1e-4   # 0.01 % of pixels


def _tolerance(g_t, g_prim, g_nx, g_ny, o_t, o_prim, o_nx, o_ny, extent=EXTENT, min_hits=1000):
    mg, mo = g_prim != lrt.MISS, o_prim != lrt.MISS
    n = g_t.size
    assert mo.sum() >= min_hits, mo.sum()
    mask = int((mg != mo).sum())
    assert mask <= FRAC * n, (mask, n)
    both = mg & mo
    dt = np.abs(g_t[both].astype(np.float64) - o_t[both])
    assert dt.max() <= 1e-4 * extent, dt.max()
    dn = np.maximum(np.abs(g_nx[both] - o_nx[both]), np.abs(g_ny[both] - o_ny[both]))
    bad = int((~(dn <= 1e-3)).sum())
    assert bad <= FRAC * n, (bad, n, float(np.nanmax(dn)))
    return dict(mask=mask, dt=float(dt.max()), normals_over=bad, exact=float((dt == 0).mean()))


def _fused_vs_oracle(s, osc, view):
    s.set_tuning("fma", 1)
    out = s.render_host([view], hits=True)["hits"]
    hits, _, _ = oracle_render(osc, view)
    return _tolerance(out["t"], out["primId"], out["nx"], out["ny"],
                      hits["t"], hits["primId"], hits["coords"][:, 2], hits["coords"][:, 3])


@pytest.mark.parametrize("intersect", [lrt.INTERSECT_NEWTON, lrt.INTERSECT_ST, lrt.INTERSECT_BBOX, lrt.INTERSECT_IT])
@pytest.mark.parametrize("depth", [4, 6])
def test_sphere_config(intersect, depth):
    h, n, v = sbs_scene(scenes.SPHERE_SDF, depth, 4)
    s = gpu_scene_sbs(h, n, v, render_mode=lrt.RENDER_MODE_NORMAL, sdf_node_intersect=intersect)
    osc = orc.Scene("sbs", sbs=(orc_header(h), n, v), intersect=intersect, render_mode=lrt.RENDER_MODE_NORMAL)
    r = _fused_vs_oracle(s, osc, scenes.sphere_view())
    s.close()
    assert r["mask"] == 0, r


@pytest.mark.parametrize("stack", [32, 64])
def test_union_scene_views(stack):
    h, n, v = lrt.sbs_from_sdf(scenes.union_sdf(), 5, 8)
    s = gpu_scene_sbs(h, n, v, render_mode=lrt.RENDER_MODE_NORMAL, sdf_node_intersect=lrt.INTERSECT_NEWTON)
    s.set_tuning("stack", stack)
    osc = orc.Scene("sbs", sbs=(orc_header(h), n, v), intersect=lrt.INTERSECT_NEWTON,
                    render_mode=lrt.RENDER_MODE_NORMAL)
    for view in scenes.union_views(n_views=3, lo=160, hi=256, cam_seed=9):
        _fused_vs_oracle(s, osc, view)
    s.close()


def test_svs_sphere():
    nodes = lrt.svs_from_sdf(lrt.Sdf(**scenes.SPHERE_SDF), 6)
    s = lrt.Scene(0)
    s.add_instance(s.add_svs(nodes))
    s.commit_scene()
    s.set_preset(render_mode=lrt.RENDER_MODE_NORMAL, sdf_node_intersect=lrt.INTERSECT_NEWTON)
    osc = orc.Scene("svs", svs=nodes, intersect=lrt.INTERSECT_NEWTON, render_mode=lrt.RENDER_MODE_NORMAL)
    _fused_vs_oracle(s, osc, scenes.sphere_view(192, 160))
    s.close()


def test_triangle_mesh_keeps_exact_kernel():
    """Triangle scenes ignore the key (a contracted edge test opens cracks
    between triangles): the records stay bit-identical."""
    verts, faces = scenes.displaced_icosphere(subdiv=5)
    s = lrt.Scene(0)
    s.add_instance(s.add_triangles(verts, faces))
    s.commit_scene()
    s.set_preset(render_mode=lrt.RENDER_MODE_NORMAL)
    view = scenes.mesh_view(width=640, height=360)
    exact = s.render_host([view], hits=True)["hits"]
    s.set_tuning("fma", 1)
    fused = s.render_host([view], hits=True)["hits"]
    s.close()
    assert (exact["primId"] != lrt.MISS).sum() > 10000
    assert np.array_equal(exact.view(np.uint32), fused.view(np.uint32))


def test_union_1024_batched_views():
    """The 1024^3 union scene (8-voxel bricks) on 4 of its 16 uneven views, one
    batched launch, contracted kernel against the bit-exact one."""
    h, n, v = lrt.sbs_from_sdf(scenes.union_sdf(), 7, 8)
    s = gpu_scene_sbs(h, n, v, render_mode=lrt.RENDER_MODE_NORMAL, sdf_node_intersect=lrt.INTERSECT_NEWTON)
    views = scenes.union_views()[:4]
    exact = s.render_host(views, hits=True)["hits"]
    s.set_tuning("fma", 1)
    fused = s.render_host(views, hits=True)["hits"]
    s.close()
    r = _tolerance(fused["t"], fused["primId"], fused["nx"], fused["ny"],
                   exact["t"], exact["primId"], exact["nx"], exact["ny"], min_hits=1000000)
    assert r["exact"] > 0.3, r


def test_tuning_key_checked():
    s = lrt.Scene(0)
    with pytest.raises(lrt.LrtError):
        s.set_tuning("fma", 2)
    s.set_tuning("fma", 0)
    s.close()
