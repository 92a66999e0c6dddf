"""GPU: scenes with several instances of one geometry (the TLAS of
RayQuery_NearestHit, BVH/BVH2Common.cpp:3508-3547; AddInstance /
UpdateInstance, BVH/BVH2Common_host.cpp:1450-1520).

The closest hit over instances does not depend on the order the instances are
walked in: a render of N instances must equal, pixel by pixel, the nearest of
N renders of one instance each (records bit-identical, the earlier instance
winning an exact tie), colours included (shaded in the frame of the instance
hit), and a batched query reports the instance in instId.  Every one of those
single-instance renders is itself bit-identical to the oracle.  UpdateInstance
on a committed multi-instance scene equals a fresh commit."""
import numpy as np
import pytest

from litert_gb300 import lrt, scenes

from _util import canon_bits

pytestmark = pytest.mark.gpu


def _mat(angle, axis, t, scale=1.0):
    a = np.asarray(axis, np.float64)
    a /= np.linalg.norm(a)
    K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    R = np.eye(3) + np.sin(angle) * K + (1 - np.cos(angle)) * K @ K
    m = np.eye(4)
    m[:3, :3] = scale * R
    m[:3, 3] = t
    return m.astype(np.float32)


MATS = [_mat(0.3, (0, 1, 0), (-0.9, 0.1, 0.0), 0.55), _mat(-0.7, (1, 1, 0), (0.8, -0.2, -0.3), 0.6),
        _mat(1.1, (0, 0, 1), (0.05, 0.75, 0.6), 0.45)]


def _scene(add, mats, preset):
    s = lrt.Scene(0)
    g = add(s)
    ids = [s.add_instance(g, m) for m in mats]
    s.commit_scene()
    s.set_preset(**preset)
    return s, ids


def _compose(parts):
    """Per pixel, the record of the nearest hit over the single-instance renders
    (strictly nearer wins: the earlier instance keeps an exact tie)."""
    best = parts[0]["hits"].copy()
    rgba = parts[0]["rgba"].copy()
    inst = np.where(best["primId"] != lrt.MISS, 0, -1)
    for k, p in enumerate(parts[1:], start=1):
        h = p["hits"]
        take = (h["primId"] != lrt.MISS) & ((best["primId"] == lrt.MISS) | (h["t"] < best["t"]))
        best[take] = h[take]
        rgba[take] = p["rgba"][take]
        inst[take] = k
    return best, rgba, inst


@pytest.mark.parametrize("kind", ["sbs", "svs", "mesh"])
def test_instances_equal_composed_single_instances(kind):
    sdf = lrt.Sdf(**scenes.union_params())
    if kind == "sbs":
        h, n, v = lrt.sbs_from_sdf(sdf, 4, 4)
        add = lambda s: s.add_sbs(h, n, v)   # noqa: E731
        preset = dict(render_mode=lrt.RENDER_MODE_LAMBERT_NO_TEX, sdf_node_intersect=lrt.INTERSECT_NEWTON)
    elif kind == "svs":
        nodes = lrt.svs_from_sdf(sdf, 5)
        add = lambda s: s.add_svs(nodes)   # noqa: E731
        preset = dict(render_mode=lrt.RENDER_MODE_NORMAL, sdf_node_intersect=lrt.INTERSECT_NEWTON)
    else:
        verts, faces = scenes.displaced_icosphere(subdiv=4)
        add = lambda s: s.add_triangles(verts, faces)   # noqa: E731
        preset = dict(render_mode=lrt.RENDER_MODE_LAMBERT_NO_TEX)
    views = scenes.union_views(n_views=2, lo=96, hi=140)
    parts = []
    for m in MATS:
        s, _ = _scene(add, [m], preset)
        parts.append(s.render_host(views, hits=True, rgba=True))
        s.close()
    want, want_rgba, want_inst = _compose(parts)
    s, ids = _scene(add, MATS, preset)
    try:
        assert ids == [0, 1, 2]
        got = s.render_host(views, hits=True, rgba=True)
        # instId of a batched query through the same pixels
        pos, dirs = [], []
        for w, hh, wv, pj in views:
            from oracle import oracle as orc
            p, d = orc.eye_rays(w, hh, lrt.inverse4x4(pj), lrt.inverse4x4(wv), np.arange(w * hh, dtype=np.uint32))
            pos.append(p)
            dirs.append(d)
        q = s.query_rays(np.concatenate(pos), np.concatenate(dirs))
    finally:
        s.close()
    hit = want["primId"] != lrt.MISS
    assert hit.sum() > 2000 and len(set(want_inst[hit].tolist())) == 3
    assert np.array_equal(canon_bits(np.ascontiguousarray(got["hits"]).view(np.float32)),
                          canon_bits(np.ascontiguousarray(want).view(np.float32)))
    assert np.array_equal(canon_bits(got["rgba"]), canon_bits(want_rgba))
    assert np.array_equal(np.where(q["primId"] != lrt.MISS, q["instId"].astype(np.int64), -1), want_inst)
    assert np.array_equal(canon_bits(q["t"][hit]), canon_bits(want["t"][hit]))


def test_update_instance_with_several_instances():
    h, n, v = lrt.sbs_from_sdf(lrt.Sdf(**scenes.union_params()), 4, 4)
    preset = dict(render_mode=lrt.RENDER_MODE_NORMAL, sdf_node_intersect=lrt.INTERSECT_NEWTON)
    views = scenes.union_views(n_views=2, lo=96, hi=128)
    moved = _mat(0.4, (1, 0, 0), (0.3, -0.6, 0.2), 0.5)
    a, _ = _scene(lambda s: s.add_sbs(h, n, v), MATS, preset)
    a.update_instance(1, moved)
    got = a.render_host(views, hits=True)["hits"]
    a.close()
    b, _ = _scene(lambda s: s.add_sbs(h, n, v), [MATS[0], moved, MATS[2]], preset)
    want = b.render_host(views, hits=True)["hits"]
    b.close()
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_instances_of_different_geometries_refused():
    h, n, v = lrt.sbs_from_sdf(scenes.sphere_sdf(), 3, 4)
    s = lrt.Scene(0)
    try:
        g0 = s.add_sbs(h, n, v)
        g1 = s.add_svs(lrt.svs_from_sdf(scenes.sphere_sdf(), 4))
        s.add_instance(g0)
        s.add_instance(g1)
        with pytest.raises(lrt.LrtError) as e:
            s.commit_scene()
        assert e.value.status == 4
    finally:
        s.close()
