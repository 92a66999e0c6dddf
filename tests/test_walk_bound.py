"""The voxel walk's step bound against rays that graze a voxel face.

The reference's brick walk (BVH/BVH2Common.cpp:764-984) has no step bound.  A
ray crosses at most 3 * brick_size voxels, but where its position rounds back
into the voxel it just left, a step advances t by the bare +1e-6: a ray nearly
parallel to a voxel face can take many such steps, running the finder in each
occupied voxel.  Engine and oracle bound the walk by 8 * brick_size + 16 steps
plus 1.5e6 per unit of the segment's length (every walk the reference finishes,
which is every walk with t < 32).  A bound of 8 * brick_size + 16 alone cut the
two rays below short and returned a farther hit; these are the first hits of the
unbounded walk.

The rays: pixels of the proposal benchmark's held-out views (16 views of 1024^2,
seed 8) of the 1024^3 smooth-union scene (depth 7, 8-voxel bricks), found by
rendering all 16.8 M pixels with and without a bound.
"""
import numpy as np
import pytest

from litert_gb300 import lrt, scenes

# (view, pixel, t and brick of the unbounded walk's closest hit)
GRAZING = [(11, 371353, 2.5415533, 48475), (12, 813364, 2.4197946, 26022)]


def _scene(gpu):
    return lrt.sbs_from_sdf(scenes.union_sdf(), 7, 8, gpu=0 if gpu else None)


def _oracle(h, nodes, values):
    from oracle import oracle as orc
    pairs = lrt.build_bvh2(orc.node_boxes(nodes), 1)
    return orc, orc.Scene("sbs", sbs=(orc.SbsHeader(h.brick_size, h.brick_pad, h.bytes_per_value, h.aux_data), nodes,
                                      values), pairs=pairs, intersect=2, render_mode=8, closest_hit=True)


def test_oracle_walks_grazing_rays_to_their_end():
    h, nodes, values = _scene(False)
    orc, osc = _oracle(h, nodes, values)
    views = scenes.proposal_views(16, 1024, seed=8)
    for vi, pix, t, prim in GRAZING:
        w, hh, wv, pj = views[vi]
        o, cnt = osc.render_pixels(w, hh, lrt.inverse4x4(pj), lrt.inverse4x4(wv), np.array([pix], np.uint32), threads=1)
        assert o["primId"][0] == prim and o["t"][0] == np.float32(t)
        # more voxel steps than 8 * brick_size + 16 (the old bound) on this ray
        assert cnt.n_vox > 8 * 8 + 16


@pytest.mark.gpu
def test_engine_walks_grazing_rays_like_the_oracle():
    h, nodes, values = _scene(True)
    orc, osc = _oracle(h, nodes, values)
    views = scenes.proposal_views(16, 1024, seed=8)
    s = lrt.Scene(0)
    try:
        s.add_instance(s.add_sbs(h, nodes, values))
        s.commit_scene()
        s.set_preset(render_mode=lrt.RENDER_MODE_NORMAL, sdf_node_intersect=lrt.INTERSECT_NEWTON)
        for vi, pix, t, prim in GRAZING:
            w, hh, wv, pj = views[vi]
            got = s.render_host([views[vi]], hits=True)["hits"][pix]
            o, _ = osc.render_pixels(w, hh, lrt.inverse4x4(pj), lrt.inverse4x4(wv), np.array([pix], np.uint32),
                                     threads=1)
            assert got["primId"] == prim and got["t"] == np.float32(t)
            assert np.array_equal(np.asarray(got).view(np.uint32)[:2], np.asarray(o[0]).view(np.uint32)[:2])
    finally:
        s.close()
