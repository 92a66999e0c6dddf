"""GPU parity of the SVS-voxel and triangle leaves against the CPU oracle
(closest hit on both sides, so the BVH topologies may differ).

SVS (OctreeNodeIntersect, BVH/BVH2Common.cpp:633-655): bit-exact hit records.
Triangles (IntersectAllTrianglesInLeaf, :2776-2840): bit-exact t, barycentrics
and normal; where a ray meets two triangles at exactly the same t (a shared
edge) the first one visited wins the strict `t < hit.t` test, so primId may
name either neighbour -- such rays must have identical t.
"""
import numpy as np
import pytest

from litert_gb300 import lrt, scenes
from oracle import oracle as orc

from _util import canon_bits, compare_hits16, oracle_render

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", [lrt.INTERSECT_NEWTON, lrt.INTERSECT_ST, lrt.INTERSECT_ANALYTIC, lrt.INTERSECT_BBOX])
def test_svs_sphere_bit_exact(mode):
    n = lrt.svs_from_sdf(lrt.Sdf(**scenes.SPHERE_SDF), 6)
    s = lrt.Scene(0)
    g = s.add_svs(n)
    s.add_instance(g)
    s.commit_scene()
    s.set_preset(render_mode=lrt.RENDER_MODE_NORMAL, sdf_node_intersect=mode)
    view = scenes.sphere_view(192, 160)
    out = s.render_host([view], hits=True, rgba=True)
    s.close()
    osc = orc.Scene("svs", svs=n, intersect=mode, render_mode=lrt.RENDER_MODE_NORMAL)
    hits, col, _ = oracle_render(osc, view)
    r = compare_hits16(out["hits"], hits)
    assert r["hits"] > 1000 and r["mask"] == 0 and r["t"] == 0 and r["prim"] == 0 and r["nx"] == 0 and r["ny"] == 0, r
    assert np.array_equal(canon_bits(out["rgba"]), canon_bits(col))


def _mesh_scene(subdiv):
    verts, faces = scenes.displaced_icosphere(subdiv=subdiv)
    s = lrt.Scene(0)
    g = s.add_triangles(verts, faces)
    s.add_instance(g)
    s.commit_scene()
    return s, verts, faces


@pytest.mark.parametrize("render_mode", [lrt.RENDER_MODE_NORMAL, lrt.RENDER_MODE_LAMBERT_NO_TEX, lrt.RENDER_MODE_DEPTH])
def test_triangles_render(render_mode):
    s, verts, faces = _mesh_scene(5)
    s.set_preset(render_mode=render_mode)
    view = scenes.mesh_view(width=320, height=180)
    out = s.render_host([view], hits=True, rgba=True)
    s.close()
    osc = orc.Scene("mesh", mesh=(verts, faces), render_mode=render_mode)
    hits, col, _ = oracle_render(osc, view)
    g = out["hits"]
    mg, mo = g["primId"] != lrt.MISS, hits["primId"] != lrt.MISS
    assert mo.sum() > 10000
    assert np.array_equal(mg, mo)
    assert np.array_equal(canon_bits(g["t"]), canon_bits(hits["t"]))
    same = g["primId"] == hits["primId"]
    assert (~same).sum() <= 1e-3 * mo.sum()           # shared-edge ties only
    assert np.array_equal(canon_bits(g["nx"][same]), canon_bits(hits["coords"][same, 2]))
    assert np.array_equal(canon_bits(g["ny"][same]), canon_bits(hits["coords"][same, 3]))
    colour_same = same | ~mo
    assert np.array_equal(canon_bits(out["rgba"][colour_same]), canon_bits(col[colour_same]))


def test_triangles_query_rays():
    s, verts, faces = _mesh_scene(4)
    s.set_preset(render_mode=lrt.RENDER_MODE_NORMAL)
    rng = np.random.default_rng(3)
    N = 20000
    pos = np.zeros((N, 4), np.float32)
    pos[:, :3] = rng.uniform(-2.5, 2.5, (N, 3))
    d = rng.normal(size=(N, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    dirs = np.zeros((N, 4), np.float32)
    dirs[:, :3] = d
    dirs[:, 3] = 1e9
    gh = s.query_rays(pos, dirs)
    s.close()
    oh = orc.Scene("mesh", mesh=(verts, faces), render_mode=lrt.RENDER_MODE_NORMAL).query_rays(pos, dirs)
    assert np.array_equal(gh["primId"] != lrt.MISS, oh["primId"] != lrt.MISS)
    assert np.array_equal(canon_bits(gh["t"]), canon_bits(oh["t"]))
    same = gh["primId"] == oh["primId"]
    assert (~same).sum() <= 1e-3 * N
    assert np.array_equal(canon_bits(gh["coords"][same]), canon_bits(oh["coords"][same]))
