"""GPU: the rest of the ISceneObject / MultiRenderer surface.

* "first_hit" tuning: renders and queries walk the BVH2 fat pairs in
  BVH2TraverseF32's order with the SDF early-out (BVH/BVH2Common.cpp:3402-3405,
  3407-3488) and equal the oracle's first-hit mode -- itself pinned to the
  reference compiled in place -- bit for bit, on the engine's own tree and on a
  caller's tree of another shape (lrt_set_bvh2), for SBS and SVS.
* RAY_GEN_MODE_RANDOM with spp 4 and a fixed seed (CastRaySingle,
  Renderer/eye_ray.cpp:100-107, rand2 :53-80): records and averaged colours
  bit-identical to the oracle's.
* UpdateInstance: a committed instance moved by a new matrix renders what a
  fresh commit with that matrix renders.
* UpdateGeom_Triangles3f: moved vertices render what a fresh commit renders;
  new connectivity is refused.
* AddGeom_AABB: refused with LRT_ERR_UNSUPPORTED.
"""
import numpy as np
import pytest

from litert_gb300 import lrt, scenes
from oracle import oracle as orc

from _util import canon_bits, records_equal

pytestmark = pytest.mark.gpu


def _median_bvh2(boxes):
    """A BVH2 of another shape than the engine's SAH tree: object-median splits
    along the widest centroid axis, one box per leaf, in the reference's fat-pair
    layout (root pair at 0, leaf payload PackOffsetAndSize(box, 1))."""
    pairs = []

    def node(ids):
        if len(ids) == 1:
            return 0x80000000 | (1 << 24) | int(ids[0]), boxes[ids[0], :3], boxes[ids[0], 3:]
        c = 0.5 * (boxes[ids, :3] + boxes[ids, 3:])
        ax = int(np.argmax(c.max(0) - c.min(0)))
        o = ids[np.argsort(c[:, ax], kind="stable")]
        me = len(pairs)
        pairs.append(None)
        lo = node(o[: len(o) // 2])
        hi = node(o[len(o) // 2:])
        pairs[me] = (lo, hi)
        return me, np.minimum(lo[1], hi[1]), np.maximum(lo[2], hi[2])

    node(np.arange(boxes.shape[0]))
    out = np.zeros(len(pairs), lrt.BVH_PAIR_DTYPE)
    for i, (l, r) in enumerate(pairs):
        out[i]["lmin"], out[i]["lleft"], out[i]["lmax"], out[i]["lesc"] = l[1], l[0], l[2], 0
        out[i]["rmin"], out[i]["rleft"], out[i]["rmax"], out[i]["resc"] = r[1], r[0], r[2], 0
    return out


def _oracle_scene(kind, data, pairs, **kw):
    if kind == "sbs":
        h, n, v = data
        return orc.Scene("sbs", sbs=(orc.SbsHeader(h.brick_size, h.brick_pad, h.bytes_per_value, h.aux_data), n, v),
                         pairs=(pairs, None, None), closest_hit=False, **kw)
    return orc.Scene("svs", svs=data, pairs=(pairs, None, None), closest_hit=False, **kw)


@pytest.mark.parametrize("kind", ["sbs", "svs"])
@pytest.mark.parametrize("tree", ["own", "median"])
def test_first_hit_walk_matches_reference_mode(kind, tree):
    sdf = lrt.Sdf(**scenes.union_params())
    if kind == "sbs":
        data = lrt.sbs_from_sdf(sdf, 5, 4)
        nodes = data[1]
    else:
        data = lrt.svs_from_sdf(sdf, 6)
        nodes = data
    s = lrt.Scene(0)
    s.add_instance(s.add_sbs(*data) if kind == "sbs" else s.add_svs(data))
    s.commit_scene()
    s.set_preset(render_mode=lrt.RENDER_MODE_NORMAL, sdf_node_intersect=lrt.INTERSECT_NEWTON)
    s.set_tuning("first_hit", 1)
    if tree == "own":
        pairs = s.bvh2()
    else:
        pairs = _median_bvh2(orc.node_boxes(nodes))
        s.set_bvh2(pairs)
    views = scenes.union_views(n_views=3, lo=96, hi=160)
    out = s.render_host(views, hits=True, rgba=True)
    rng = np.random.default_rng(5)
    N = 6000
    pos = np.zeros((N, 4), np.float32)
    pos[:, :3] = rng.uniform(-2.5, 2.5, (N, 3))
    d = rng.normal(size=(N, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    dirs = np.zeros((N, 4), np.float32)
    dirs[:, :3] = d
    dirs[:, 3] = 1e9
    q = s.query_rays(pos, dirs)
    s.set_tuning("first_hit", 0)
    closest = s.render_host(views, hits=True)["hits"]
    s.close()
    osc = _oracle_scene(kind, data, pairs, intersect=lrt.INTERSECT_NEWTON, render_mode=lrt.RENDER_MODE_NORMAL)
    off = 0
    differs = 0
    for w, hh, wv, pj in views:
        o, col, _ = osc.render(w, hh, lrt.inverse4x4(pj), lrt.inverse4x4(wv), rgba=True)
        g = out["hits"][off:off + w * hh]
        assert np.array_equal(g["primId"], o["primId"])
        hit = o["primId"] != lrt.MISS
        assert hit.sum() > 500
        for f, c in (("t", None), ("nx", 2), ("ny", 3)):
            ov = o["t"] if c is None else o["coords"][:, c]
            assert np.array_equal(canon_bits(g[f][hit]), canon_bits(ov[hit])), f
        assert np.array_equal(canon_bits(out["rgba"][off:off + w * hh]), canon_bits(col))
        differs += int((closest["t"][off:off + w * hh] != g["t"]).sum())
        off += w * hh
    oq = osc.query_rays(pos, dirs)
    assert records_equal(q, oq)
    print(f"{kind}/{tree}: first-hit records differ from the closest hit on {differs} of {off} pixels")


def test_random_ray_generation_spp4():
    h, n, v = lrt.sbs_from_sdf(scenes.sphere_sdf(), 4, 4)
    s = lrt.Scene(0)
    s.add_instance(s.add_sbs(h, n, v))
    s.commit_scene()
    s.set_seed(12345)
    s.set_preset(render_mode=lrt.RENDER_MODE_LAMBERT_NO_TEX, sdf_node_intersect=lrt.INTERSECT_NEWTON, spp=4,
                 ray_gen_mode=1)
    view = scenes.sphere_view(96, 80)
    out = s.render_host([view], hits=True, rgba=True)
    s.set_seed(7)
    other = s.render_host([view], rgba=True)["rgba"]
    s.set_preset(ray_gen_mode=0)
    regular = s.render_host([view], rgba=True)["rgba"]
    s.close()
    osc = orc.Scene("sbs", sbs=(orc.SbsHeader(h.brick_size, h.brick_pad, h.bytes_per_value, h.aux_data), n, v),
                    intersect=lrt.INTERSECT_NEWTON, render_mode=lrt.RENDER_MODE_LAMBERT_NO_TEX, spp=4,
                    ray_gen_mode=1, seed=12345)
    w, hh, wv, pj = view
    o, col, _ = osc.render(w, hh, lrt.inverse4x4(pj), lrt.inverse4x4(wv), rgba=True)
    g = out["hits"]
    assert np.array_equal(g["primId"], o["primId"])
    hit = o["primId"] != lrt.MISS
    assert np.array_equal(canon_bits(g["t"][hit]), canon_bits(o["t"][hit]))
    assert np.array_equal(canon_bits(out["rgba"]), canon_bits(col))
    # the offsets really are random: another seed and the regular grid give other edge colours
    assert not np.array_equal(out["rgba"], other)
    assert not np.array_equal(out["rgba"], regular)


def test_update_instance_equals_fresh_commit():
    h, n, v = lrt.sbs_from_sdf(lrt.Sdf(**scenes.union_params()), 5, 4)
    m = np.eye(4, dtype=np.float32)
    m[:3, :3] = np.array([[0.8, -0.6, 0], [0.6, 0.8, 0], [0, 0, 1]], np.float32)
    m[:3, 3] = [0.2, -0.1, 0.3]
    views = scenes.union_views(n_views=2, lo=96, hi=128)
    a = lrt.Scene(0)
    g = a.add_sbs(h, n, v)
    iid = a.add_instance(g)
    a.commit_scene()
    a.set_preset(render_mode=lrt.RENDER_MODE_NORMAL, sdf_node_intersect=lrt.INTERSECT_NEWTON)
    before = a.render_host(views, hits=True)["hits"]
    a.update_instance(iid, m)
    moved = a.render_host(views, hits=True)["hits"]
    a.close()
    b = lrt.Scene(0)
    b.add_instance(b.add_sbs(h, n, v), m)
    b.commit_scene()
    b.set_preset(render_mode=lrt.RENDER_MODE_NORMAL, sdf_node_intersect=lrt.INTERSECT_NEWTON)
    fresh = b.render_host(views, hits=True)["hits"]
    b.close()
    assert records_equal(moved, fresh)
    assert not records_equal(moved, before)


def test_update_geom_triangles_and_aabb():
    verts, faces = scenes.displaced_icosphere(subdiv=4)
    moved = (verts * np.float32(1.1)).astype(np.float32)
    view = scenes.mesh_view(width=160, height=120)
    a = lrt.Scene(0)
    g = a.add_triangles(verts, faces)
    a.add_instance(g)
    a.commit_scene()
    a.set_preset(render_mode=lrt.RENDER_MODE_NORMAL)
    a.update_geom_triangles(g, moved)
    got = a.render_host([view], hits=True)["hits"]
    with pytest.raises(lrt.LrtError) as e:
        a.update_geom_triangles(g, moved, faces[::-1].copy())
    assert e.value.status == 4
    with pytest.raises(lrt.LrtError) as e:
        a.add_aabb(np.zeros((3, 8), np.float32))
    assert e.value.status == 4
    a.close()
    b = lrt.Scene(0)
    b.add_instance(b.add_triangles(moved, faces))
    b.commit_scene()
    b.set_preset(render_mode=lrt.RENDER_MODE_NORMAL)
    fresh = b.render_host([view], hits=True)["hits"]
    b.close()
    hit = fresh["primId"] != lrt.MISS
    assert hit.sum() > 1000
    assert np.array_equal(got["primId"] != lrt.MISS, hit)
    assert np.array_equal(canon_bits(got["t"][hit]), canon_bits(fresh["t"][hit]))


def test_set_bvh2_rejects_malformed_trees():
    h, n, v = lrt.sbs_from_sdf(scenes.sphere_sdf(), 4, 4)
    s = lrt.Scene(0)
    s.add_instance(s.add_sbs(h, n, v))
    s.commit_scene()
    good = s.bvh2()
    bad_leaf = good.copy()
    leaf = np.flatnonzero(bad_leaf["lleft"] & 0x80000000)[0]
    bad_leaf[leaf]["lleft"] = 0x80000000 | (1 << 24) | (n.shape[0] + 5)      # brick out of range
    cyc = good.copy()
    inner = np.flatnonzero((cyc["lleft"] & 0x80000000) == 0)[0]
    cyc[inner]["lleft"] = 0                                                   # back to the root
    try:
        for bad in (bad_leaf, cyc):
            with pytest.raises(lrt.LrtError) as e:
                s.set_bvh2(bad)
            assert e.value.status == 1
        s.set_bvh2(good)
    finally:
        s.close()
