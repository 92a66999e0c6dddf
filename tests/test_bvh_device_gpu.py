"""BVH built on the device (lrt_set_tuning "bvh_builder" 1: binned SAH, 2: linear
BVH) and triangle refit.

The device SAH builder restates the host builder level by level, so its tree is
the host's: the fat pairs are byte-identical and renders bit-identical.  The
linear BVH (Morton codes, radix sort, radix tree, 4-wide collapse) has another
topology, so the closest hit is compared, not the tree: every leaf box is the
primitive's box either way, so hit masks and t are bit-identical; the primitive
may differ only where a ray meets two primitives at exactly the same t (a shared
edge or brick face), and there the records must agree in t.  Refit keeps the topology and
recomputes the boxes: a refit with unchanged vertices reproduces the committed
boxes bit for bit, and a refit to moved vertices renders what a fresh build of
the moved mesh renders.
"""
import numpy as np
import pytest

from litert_gb300 import lrt, scenes
from oracle import oracle as orc

from _util import canon_bits, compare_hits16, oracle_render, records_equal

pytestmark = pytest.mark.gpu


def _render(scene, views, **kw):
    return scene.render_host(views, **kw)


def _sbs_scene(builder, h, nodes, values, mode=lrt.INTERSECT_ST, render_mode=lrt.RENDER_MODE_NORMAL):
    s = lrt.Scene(0)
    s.set_tuning("bvh_builder", builder)
    g = s.add_sbs(h, nodes, values)
    s.add_instance(g)
    s.commit_scene()
    s.set_preset(render_mode=render_mode, sdf_node_intersect=mode)
    return s


def _same_closest_hits(a, b, tie_frac=1e-4):
    ma, mb = a["primId"] != lrt.MISS, b["primId"] != lrt.MISS
    assert np.array_equal(ma, mb)
    assert np.array_equal(canon_bits(a["t"]), canon_bits(b["t"]))
    same = a["primId"] == b["primId"]
    assert (~same).sum() <= max(2, tie_frac * ma.sum())
    assert records_equal(a[same], b[same])
    return int(ma.sum())


@pytest.mark.parametrize("builder", [1, 2])
@pytest.mark.parametrize("mode", [lrt.INTERSECT_ST, lrt.INTERSECT_NEWTON])
def test_device_bvh_sbs_matches_host(mode, builder):
    h, nodes, values = lrt.sbs_from_sdf(scenes.union_sdf(), 6, 4)
    views = scenes.union_views(n_views=3, lo=96, hi=200)
    outs = []
    for builder in (0, builder):
        s = _sbs_scene(builder, h, nodes, values, mode)
        outs.append(_render(s, views, hits=True, rgba=True))
        s.close()
    n = _same_closest_hits(outs[0]["hits"], outs[1]["hits"])
    assert n > 5000
    same = outs[0]["hits"]["primId"] == outs[1]["hits"]["primId"]
    assert np.array_equal(canon_bits(outs[0]["rgba"][same]), canon_bits(outs[1]["rgba"][same]))


@pytest.mark.parametrize("builder", [1, 2])
def test_device_bvh_sbs_matches_oracle(builder):
    h, nodes, values = lrt.sbs_from_sdf(scenes.sphere_sdf(), 5, 4)
    s = _sbs_scene(builder, h, nodes, values)
    view = scenes.sphere_view(160, 128)
    out = _render(s, [view], hits=True)
    s.close()
    osc = orc.Scene("sbs", sbs=(orc.SbsHeader(h.brick_size, h.brick_pad, h.bytes_per_value, h.aux_data), nodes, values),
                    intersect=lrt.INTERSECT_ST, render_mode=lrt.RENDER_MODE_NORMAL)
    hits, _, _ = oracle_render(osc, view)
    r = compare_hits16(out["hits"], hits)
    assert r["hits"] > 1000 and r["mask"] == 0 and r["t"] == 0, r


@pytest.mark.parametrize("builder", [1, 2])
def test_device_bvh_svs_matches_host(builder):
    n = lrt.svs_from_sdf(scenes.union_sdf(), 6)
    view = scenes.union_views(n_views=1, lo=160, hi=161)
    outs = []
    for builder in (0, builder):
        s = lrt.Scene(0)
        s.set_tuning("bvh_builder", builder)
        g = s.add_svs(n)
        s.add_instance(g)
        s.commit_scene()
        s.set_preset(render_mode=lrt.RENDER_MODE_NORMAL)
        outs.append(_render(s, view, hits=True)["hits"])
        s.close()
    assert _same_closest_hits(outs[0], outs[1]) > 2000


@pytest.mark.parametrize("builder", [1, 2])
@pytest.mark.parametrize("n_bricks", [1, 2, 3, 5])
def test_device_bvh_tiny_scenes(n_bricks, builder):
    h, nodes, values = lrt.sbs_from_sdf(scenes.sphere_sdf(), 3, 4)
    nodes = nodes[:n_bricks].copy()
    view = scenes.sphere_view(128, 128)
    outs = []
    for builder in (0, builder):
        s = _sbs_scene(builder, h, nodes, values)
        outs.append(_render(s, [view], hits=True)["hits"])
        s.close()
    _same_closest_hits(outs[0], outs[1])


def _pairs_of(builder, h, nodes, values):
    s = _sbs_scene(builder, h, nodes, values)
    p = s.bvh2()
    s.close()
    return p


@pytest.mark.parametrize("depth,brick", [(5, 4), (7, 8), (4, 2)])
def test_device_sah_is_the_host_tree(depth, brick):
    h, nodes, values = lrt.sbs_from_sdf(scenes.union_sdf(), depth, brick)
    host = _pairs_of(0, h, nodes, values)
    dev = _pairs_of(1, h, nodes, values)
    assert host.shape == dev.shape and host.tobytes() == dev.tobytes()


@pytest.mark.parametrize("depth", [5, 7])
def test_device_sah_svs_is_the_host_tree(depth):
    n = lrt.svs_from_sdf(scenes.union_sdf(), depth)
    pairs = []
    for builder in (0, 1):
        s = lrt.Scene(0)
        s.set_tuning("bvh_builder", builder)
        g = s.add_svs(n)
        s.add_instance(g)
        s.commit_scene()
        pairs.append(s.bvh2())
        s.close()
    assert pairs[0].tobytes() == pairs[1].tobytes()


@pytest.mark.parametrize("subdiv", [4, 6])   # 6: 81,920 triangles, the top levels split by many blocks
def test_device_sah_mesh_is_the_host_tree(subdiv):
    verts, faces = scenes.displaced_icosphere(subdiv=subdiv)
    view = scenes.mesh_view(width=240, height=160)
    a = _mesh_render(verts, faces, 0, view, pairs=True)
    b = _mesh_render(verts, faces, 1, view, pairs=True)
    assert a["pairs"].tobytes() == b["pairs"].tobytes()
    assert records_equal(a["hits"], b["hits"])
    assert np.array_equal(canon_bits(a["rgba"]), canon_bits(b["rgba"]))


@pytest.mark.parametrize("builder", [1, 2])
def test_device_bvh_fat_pairs_cover_every_brick(builder):
    h, nodes, values = lrt.sbs_from_sdf(scenes.union_sdf(), 5, 4)
    s = _sbs_scene(builder, h, nodes, values)
    p = s.bvh2()
    s.close()
    nb = nodes.shape[0]
    assert p.shape[0] == max(1, nb - 1)   # one brick per leaf either way
    seen = np.zeros(nb, np.int64)
    # walk from the root pair: every pair reached once, child boxes inside the parent box
    stack = [(0, None)]
    reached = np.zeros(p.shape[0], np.int64)
    while stack:
        i, parent_box = stack.pop()
        reached[i] += 1
        for side in ("l", "r"):
            lo, hi, ref = p[i][side + "min"], p[i][side + "max"], int(p[i][side + "left"])
            if parent_box is not None:
                assert np.all(lo >= parent_box[0]) and np.all(hi <= parent_box[1])
            if ref & 0x80000000:
                assert (ref >> 24) & 0x7F == 1
                seen[ref & 0x00FFFFFF] += 1
            else:
                stack.append((ref, (lo, hi)))
    assert np.all(reached == 1)
    assert np.all(seen == 1)


def _moved(verts, seed):
    rng = np.random.default_rng(seed)
    v = verts.astype(np.float32).copy()
    v[:, :3] = v[:, :3] * np.float32(0.85) + rng.normal(0, 0.01, (v.shape[0], 3)).astype(np.float32)
    v[:, :3] += np.float32([0.1, -0.05, 0.02])
    return v


def _mesh_render(verts, faces, builder, view, refit_to=None, pairs=False):
    s = lrt.Scene(0)
    s.set_tuning("bvh_builder", builder)
    g = s.add_triangles(verts, faces)
    s.add_instance(g)
    s.commit_scene()
    s.set_preset(render_mode=lrt.RENDER_MODE_NORMAL)
    pr = s.bvh2() if pairs else None
    if refit_to is not None:
        s.refit_triangles(refit_to)
    out = _render(s, [view], hits=True, rgba=True)
    s.close()
    if pairs:
        out["pairs"] = pr
    return out


@pytest.mark.parametrize("builder", [0, 1, 2])
def test_device_bvh_mesh_matches_oracle(builder):
    verts, faces = scenes.displaced_icosphere(subdiv=4)
    view = scenes.mesh_view(width=240, height=160)
    out = _mesh_render(verts, faces, builder, view)
    osc = orc.Scene("mesh", mesh=(verts, faces), render_mode=lrt.RENDER_MODE_NORMAL)
    hits, _, _ = oracle_render(osc, view)
    g = out["hits"]
    mg, mo = g["primId"] != lrt.MISS, hits["primId"] != lrt.MISS
    assert mo.sum() > 5000 and np.array_equal(mg, mo)
    assert np.array_equal(canon_bits(g["t"]), canon_bits(hits["t"]))
    assert (g["primId"] != hits["primId"]).sum() <= 1e-3 * mo.sum()


@pytest.mark.parametrize("builder", [0, 1, 2])
def test_refit_unchanged_is_identity(builder):
    verts, faces = scenes.displaced_icosphere(subdiv=4)
    view = scenes.mesh_view(width=240, height=160)
    a = _mesh_render(verts, faces, builder, view)
    b = _mesh_render(verts, faces, builder, view, refit_to=verts)
    assert records_equal(a["hits"], b["hits"])
    assert np.array_equal(canon_bits(a["rgba"]), canon_bits(b["rgba"]))


@pytest.mark.parametrize("builder", [0, 1, 2])
def test_refit_moved_matches_fresh_build(builder):
    verts, faces = scenes.displaced_icosphere(subdiv=4)
    moved = _moved(verts, 7)
    view = scenes.mesh_view(width=240, height=160)
    refit = _mesh_render(verts, faces, builder, view, refit_to=moved)
    fresh = _mesh_render(moved, faces, 0, view)
    g, f = refit["hits"], fresh["hits"]
    mg, mf = g["primId"] != lrt.MISS, f["primId"] != lrt.MISS
    assert mf.sum() > 3000 and np.array_equal(mg, mf)
    assert np.array_equal(canon_bits(g["t"]), canon_bits(f["t"]))
    same = g["primId"] == f["primId"]
    assert (~same).sum() <= 1e-3 * mf.sum()
    assert records_equal(g[same], f[same])


def test_refit_rejects_bad_input_and_blocks_stale_pairs():
    verts, faces = scenes.displaced_icosphere(subdiv=2)
    s = lrt.Scene(0)
    g = s.add_triangles(verts, faces)
    s.add_instance(g)
    s.commit_scene()
    with pytest.raises(lrt.LrtError):
        s.refit_triangles(verts[:-1])
    s.refit_triangles(verts)
    with pytest.raises(lrt.LrtError):
        s.bvh2()
    s.close()
    h, nodes, values = lrt.sbs_from_sdf(scenes.sphere_sdf(), 3, 4)
    s = _sbs_scene(0, h, nodes, values)
    with pytest.raises(lrt.LrtError):
        s.refit_triangles(verts)
    s.close()
