"""GPU: kernel_RayTrace's shading modes (Renderer/eye_ray.cpp:162-489) against the
oracle: palette modes (PRIMITIVE / TYPE / GEOM), BARYCENTRIC, ST_ITERATIONS,
DIFFUSE, LAMBERT with the default material, HSV_DEPTH bit for bit; PHONG and
PHONG_NO_TEX, whose direct light casts a shadow ray, to 1e-5 (the specular term's
powf may differ from glibc's in the last place); the radiance-field, splat and
texture-coordinate modes are refused."""
import numpy as np
import pytest

from litert_gb300 import lrt, scenes
from oracle import oracle as orc

from _util import canon_bits, gpu_scene_sbs, orc_header, oracle_render, sbs_scene

pytestmark = pytest.mark.gpu

EXACT = [lrt.RENDER_MODE_PRIMITIVE, lrt.RENDER_MODE_TYPE, lrt.RENDER_MODE_GEOM, lrt.RENDER_MODE_BARYCENTRIC,
         lrt.RENDER_MODE_DIFFUSE, lrt.RENDER_MODE_LAMBERT, lrt.RENDER_MODE_HSV_DEPTH]


def _sbs(params, depth, bs, mode, intersect=lrt.INTERSECT_NEWTON):
    h, n, v = sbs_scene(params, depth, bs)
    g = gpu_scene_sbs(h, n, v, render_mode=mode, sdf_node_intersect=intersect)
    osc = orc.Scene("sbs", sbs=(orc_header(h), n, v), intersect=intersect, render_mode=mode)
    return g, osc


@pytest.mark.parametrize("mode", EXACT)
def test_sbs_modes_bit_exact(mode):
    g, osc = _sbs(scenes.SPHERE_SDF, 4, 4, mode)
    view = scenes.sphere_view(96, 80)
    out = g.render_host([view], hits=True, rgba=True)
    g.close()
    _, col, _ = oracle_render(osc, view)
    assert (out["hits"]["primId"] != lrt.MISS).sum() > 300
    assert np.array_equal(canon_bits(out["rgba"]), canon_bits(col))


@pytest.mark.parametrize("intersect", [lrt.INTERSECT_ST, lrt.INTERSECT_IT])
def test_st_iterations_mode(intersect):
    g, osc = _sbs(scenes.SPHERE_SDF, 4, 4, lrt.RENDER_MODE_ST_ITERATIONS, intersect)
    view = scenes.sphere_view(96, 80)
    out = g.render_host([view], hits=True, rgba=True)
    g.close()
    hits, col, _ = oracle_render(osc, view)
    assert np.array_equal(out["hits"]["primId"], hits["primId"])   # iteration counts
    assert np.array_equal(canon_bits(out["rgba"]), canon_bits(col))
    assert len(np.unique(out["rgba"][:, 1])) > 3


@pytest.mark.parametrize("mode", [lrt.RENDER_MODE_PHONG_NO_TEX, lrt.RENDER_MODE_PHONG])
def test_phong_with_shadows(mode):
    h, n, v = lrt.sbs_from_sdf(scenes.union_sdf(), 5, 8)
    g = gpu_scene_sbs(h, n, v, render_mode=mode, sdf_node_intersect=lrt.INTERSECT_NEWTON)
    osc = orc.Scene("sbs", sbs=(orc_header(h), n, v), intersect=lrt.INTERSECT_NEWTON, render_mode=mode)
    for view in scenes.union_views(n_views=2, lo=128, hi=192, cam_seed=4):
        out = g.render_host([view], hits=True, rgba=True)
        _, col, _ = oracle_render(osc, view)
        hit = out["hits"]["primId"] != lrt.MISS
        assert hit.sum() > 1000
        assert np.abs(out["rgba"] - col).max() <= 1e-5
        # shadows present: lit pixels facing the light are brighter than shadowed ones
        assert len(np.unique(np.round(out["rgba"][hit, 1], 3))) > 10
    g.close()


def _mesh(subdiv=4):
    verts, faces = scenes.displaced_icosphere(subdiv=subdiv)
    s = lrt.Scene(0)
    s.add_instance(s.add_triangles(verts, faces))
    s.commit_scene()
    return s, verts, faces


@pytest.mark.parametrize("mode", [lrt.RENDER_MODE_PRIMITIVE, lrt.RENDER_MODE_BARYCENTRIC, lrt.RENDER_MODE_GEOM,
                                  lrt.RENDER_MODE_PHONG_NO_TEX, lrt.RENDER_MODE_LAMBERT])
def test_triangle_modes(mode):
    s, verts, faces = _mesh()
    s.set_preset(render_mode=mode)
    view = scenes.mesh_view(width=256, height=160)
    out = s.render_host([view], hits=True, rgba=True)
    s.close()
    osc = orc.Scene("mesh", mesh=(verts, faces), render_mode=mode)
    hits, col, _ = oracle_render(osc, view)
    same = (out["hits"]["primId"] == hits["primId"])   # closest-hit ties on shared edges aside
    assert same.mean() > 0.999
    tol = 1e-5 if mode == lrt.RENDER_MODE_PHONG_NO_TEX else 0.0
    assert np.abs(out["rgba"][same] - col[same]).max() <= tol


@pytest.mark.parametrize("mode", [11, 13, 14, 15, 20])
def test_unsupported_modes_refused(mode):
    s = lrt.Scene(0)
    with pytest.raises(lrt.LrtError):
        s.set_preset(render_mode=mode)
    s.close()
