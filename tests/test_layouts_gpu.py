"""GPU: coloured (DX_RGB8) and textured (DX_UV16) brick sets of
tests/golden/ref_layouts.npz.  The engine's closest-hit records on the reference
rays equal the oracle's bit for bit (distance, brick, colour or texture
coordinates, normal, type bits 11 / 10), and the DIFFUSE and BARYCENTRIC images
(which show the colour and the texture coordinates) equal the oracle's."""
import os

import numpy as np
import pytest

from litert_gb300 import lrt, scenes
from oracle import oracle as orc

from _util import canon_bits, oracle_render

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden", "ref_layouts.npz")
RAYS = os.path.join(HERE, "golden", "ref_rayquery.npz")


def _case(name):
    g = np.load(GOLD)
    hdr = [int(x) for x in g[name + "_hdr"]]
    return lrt.SbsHeader(*hdr), orc.SbsHeader(*hdr), g[name + "_nodes"], g[name + "_values"]


@pytest.mark.parametrize("name,type_bits", [("rgb8_q4", 11), ("rgb8_q1pad", 11), ("uv16_q2", 10)])
def test_layout_records(name, type_bits):
    h, oh, n, v = _case(name)
    r = np.load(RAYS)
    s = lrt.Scene(0)
    s.add_instance(s.add_sbs(h, n, v))
    s.commit_scene()
    s.set_preset(render_mode=lrt.RENDER_MODE_NORMAL, sdf_node_intersect=lrt.INTERSECT_NEWTON)
    got = s.query_rays(r["rays_pos"], r["rays_dir"])
    s.close()
    want = orc.Scene("sbs", sbs=(oh, n, v), intersect=2, render_mode=8).query_rays(r["rays_pos"], r["rays_dir"])
    hit = want["primId"] != lrt.MISS
    assert hit.sum() > 300
    assert np.all((got["geomId"][hit] >> 24) == type_bits)
    for f in ("t", "primId", "geomId"):
        assert np.array_equal(got[f], want[f]), f
    assert np.array_equal(canon_bits(got["coords"][hit]), canon_bits(want["coords"][hit]))


@pytest.mark.parametrize("name,mode", [("rgb8_q4", lrt.RENDER_MODE_DIFFUSE), ("rgb8_q1pad", lrt.RENDER_MODE_LAMBERT),
                                       ("uv16_q2", lrt.RENDER_MODE_BARYCENTRIC)])
def test_layout_images(name, mode):
    h, oh, n, v = _case(name)
    s = lrt.Scene(0)
    s.add_instance(s.add_sbs(h, n, v))
    s.commit_scene()
    s.set_preset(render_mode=mode, sdf_node_intersect=lrt.INTERSECT_NEWTON)
    view = scenes.union_views(n_views=1, lo=160, hi=200, cam_seed=2)[0]
    out = s.render_host([view], hits=True, rgba=True)
    s.close()
    _, col, _ = oracle_render(orc.Scene("sbs", sbs=(oh, n, v), intersect=2, render_mode=mode), view)
    assert (out["hits"]["primId"] != lrt.MISS).sum() > 1000
    assert np.array_equal(canon_bits(out["rgba"]), canon_bits(col))
    assert len(np.unique(out["rgba"][:, 0])) > 20   # the colours / coordinates vary


@pytest.mark.parametrize("normal_mode", [0, 2])
def test_smoothed_normals(normal_mode):
    """NORMAL_MODE_SDF_SMOOTHED on the neighbour layout: query records and NORMAL /
    LAMBERT images equal the oracle's (which equals the reference's) bit for bit."""
    g = np.load(GOLD)
    r = np.load(RAYS)
    hdr = [int(x) for x in g["smooth_hdr"]]
    h, oh = lrt.SbsHeader(*hdr), orc.SbsHeader(*hdr)
    n, v, vf = g["smooth_nodes"], g["smooth_values"], g["smooth_values_f"]
    s = lrt.Scene(0)
    s.add_instance(s.add_sbs(h, n, v, vf))
    s.commit_scene()
    s.set_preset(render_mode=lrt.RENDER_MODE_NORMAL, sdf_node_intersect=lrt.INTERSECT_NEWTON, normal_mode=normal_mode)
    got = s.query_rays(r["rays_pos"], r["rays_dir"])
    osc = orc.Scene("sbs", sbs=(oh, n, v, vf), intersect=2, render_mode=8, normal_mode=normal_mode)
    want = osc.query_rays(r["rays_pos"], r["rays_dir"])
    hit = want["primId"] != lrt.MISS
    assert hit.sum() > 300
    assert np.array_equal(got["primId"], want["primId"]) and np.array_equal(got["t"], want["t"])
    assert np.array_equal(canon_bits(got["coords"][hit]), canon_bits(want["coords"][hit]))
    for mode in (lrt.RENDER_MODE_NORMAL, lrt.RENDER_MODE_LAMBERT):
        s.set_preset(render_mode=mode, sdf_node_intersect=lrt.INTERSECT_NEWTON, normal_mode=normal_mode)
        view = scenes.union_views(n_views=1, lo=128, hi=160, cam_seed=5)[0]
        out = s.render_host([view], hits=True, rgba=True)
        _, col, _ = oracle_render(orc.Scene("sbs", sbs=(oh, n, v, vf), intersect=2, render_mode=mode,
                                            normal_mode=normal_mode), view)
        assert np.array_equal(canon_bits(out["rgba"]), canon_bits(col))
    s.close()
