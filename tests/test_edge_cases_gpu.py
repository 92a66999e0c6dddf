"""GPU edge cases of the forward path against the oracle: ragged and one-pixel
views (tiles cut by the image border), a camera inside the brick set, views that
miss everything, degenerate triangles, the largest accepted view, and a batch of
many small uneven views equal to the same views rendered one by one."""
import numpy as np
import pytest

from litert_gb300 import lrt, scenes
from oracle import oracle as orc

from _util import canon_bits, compare_hits16, gpu_scene_sbs, oracle_render, orc_header, records_equal, sbs_scene

pytestmark = pytest.mark.gpu


def _sphere_scene():
    h, n, v = sbs_scene(scenes.SPHERE_SDF, 5, 4)
    s = gpu_scene_sbs(h, n, v, render_mode=lrt.RENDER_MODE_NORMAL, sdf_node_intersect=lrt.INTERSECT_NEWTON)
    osc = orc.Scene("sbs", sbs=(orc_header(h), n, v), intersect=lrt.INTERSECT_NEWTON,
                    render_mode=lrt.RENDER_MODE_NORMAL)
    return s, osc


@pytest.mark.parametrize("w,h", [(1, 1), (1, 37), (37, 1), (13, 7), (33, 65)])
def test_ragged_and_tiny_views(w, h):
    s, osc = _sphere_scene()
    view = scenes.camera((0.1, 0.2, 2.0), (0, 0, 0), (0, 1, 0), 40.0, w, h)
    out = s.render_host([view], hits=True)["hits"]
    s.close()
    hits, _, _ = oracle_render(osc, view)
    r = compare_hits16(out, hits)
    assert r["mask"] == 0 and r["t"] == 0 and r["prim"] == 0 and r["nx"] == 0 and r["ny"] == 0, r


def test_camera_inside_the_brick_set():
    s, osc = _sphere_scene()
    view = scenes.camera((0.0, 0.0, 0.0), (0.3, 0.1, 1.0), (0, 1, 0), 90.0, 64, 48)   # at the sphere's centre
    out = s.render_host([view], hits=True)["hits"]
    s.close()
    hits, _, _ = oracle_render(osc, view)
    r = compare_hits16(out, hits)
    assert r["hits"] > 1000 and r["mask"] == 0 and r["t"] == 0 and r["prim"] == 0, r


def test_view_missing_everything():
    s, osc = _sphere_scene()
    view = scenes.camera((0, 0, 3), (0, 0, 6), (0, 1, 0), 30.0, 40, 30)   # looking away
    out = s.render_host([view], hits=True, rgba=True)
    s.close()
    assert np.all(out["hits"]["primId"] == lrt.MISS)
    hits, col, _ = oracle_render(osc, view)
    assert np.all(hits["primId"] == lrt.MISS)
    assert np.array_equal(canon_bits(out["rgba"]), canon_bits(col))


def test_degenerate_triangles():
    verts, faces = scenes.displaced_icosphere(subdiv=3)
    verts = np.asarray(verts, np.float32)
    faces = np.asarray(faces, np.uint32).reshape(-1, 3).copy()
    rng = np.random.default_rng(4)
    pick = rng.choice(faces.shape[0], 60, replace=False)
    faces[pick[:30], 2] = faces[pick[:30], 1]                    # two equal vertices: zero area
    extra = np.repeat(faces[pick[30:], :1], 3, axis=1)            # a triangle collapsed to a point
    faces = np.concatenate([faces, extra], 0)
    s = lrt.Scene(0)
    g = s.add_triangles(verts, faces)
    s.add_instance(g)
    s.commit_scene()
    s.set_preset(render_mode=lrt.RENDER_MODE_NORMAL)
    view = scenes.mesh_view(width=160, height=120)
    out = s.render_host([view], hits=True)["hits"]
    s.close()
    osc = orc.Scene("mesh", mesh=(verts, faces), render_mode=lrt.RENDER_MODE_NORMAL)
    hits, _, _ = oracle_render(osc, view)
    mg, mo = out["primId"] != lrt.MISS, hits["primId"] != lrt.MISS
    assert mo.sum() > 1000 and np.array_equal(mg, mo)
    assert np.array_equal(canon_bits(out["t"]), canon_bits(hits["t"]))


def test_largest_view_accepted_and_beyond_refused():
    s, osc = _sphere_scene()
    # 65535 x 1 (16-bit image coordinates): the row spans a very wide horizontal
    # field, the sphere covers a few pixels of it
    view = scenes.camera((0, 0, 3), (0, 0, 0), (0, 1, 0), 60.0, 65535, 1)
    out = s.render_host([view], hits=True)["hits"]
    hits, _, _ = oracle_render(osc, view)
    r = compare_hits16(out, hits)
    assert r["hits"] >= 1 and r["mask"] == 0 and r["t"] == 0 and r["prim"] == 0, r
    with pytest.raises(lrt.LrtError):
        s.render_host([scenes.camera((0, 0, 3), (0, 0, 0), (0, 1, 0), 60.0, 65536, 1)])
    s.close()


def test_many_uneven_views_in_one_launch():
    s, _ = _sphere_scene()
    rng = np.random.default_rng(11)
    views = []
    for i in range(48):
        a = rng.uniform(0, 2 * np.pi)
        views.append(scenes.camera((2.5 * np.sin(a), rng.uniform(-1, 1), 2.5 * np.cos(a)), (0, 0, 0), (0, 1, 0),
                                rng.uniform(30, 70), int(rng.integers(1, 90)), int(rng.integers(1, 90))))
    batched = s.render_host(views, hits=True)["hits"]
    off = 0
    for v in views:
        single = s.render_host([v], hits=True)["hits"]
        assert records_equal(batched[off:off + single.size], single)
        off += single.size
    assert off == batched.size
    s.close()
