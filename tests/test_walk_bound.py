"""The voxel walk's step bound against rays that graze a voxel face.

The reference's brick walk (BVH/BVH2Common.cpp:764-984) has no step bound.  A
ray crosses at most 3 * brick_size voxels, but where its position rounds back
into the voxel it just left, a step advances t by the bare +1e-6: a ray nearly
parallel to a voxel face can take many such steps, running the finder in each
occupied voxel.  Engine and oracle bound the walk by 8 * brick_size + 16 steps
plus 1.5e6 per unit of the segment's length (every walk the reference finishes,
which is every walk with t < 32).  A bound of 8 * brick_size + 16 alone cut the
two rays below short and returned a farther hit.

The rays: pixels of the proposal benchmark's held-out views (16 views of 1024^2,
seed 8) of the 1024^3 smooth-union scene (depth 7, 8-voxel bricks), found by
rendering all 16.8 M pixels with and without a bound.  tests/golden/
walk_bound_grazing.npz (tests/golden/make_golden_walk_bound.py) holds the 40
bricks they cross and the closest hits of a walk without a bound.
"""
import os

import numpy as np
import pytest

from litert_gb300 import lrt, scenes

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "walk_bound_grazing.npz"))


def _fixture():
    h = lrt.SbsHeader(*[int(x) for x in GOLD["header"]])
    return h, GOLD["nodes"], GOLD["values"]


def _oracle(h, nodes, values):
    from oracle import oracle as orc
    pairs = lrt.build_bvh2(orc.node_boxes(nodes), 1)
    return orc.Scene("sbs", sbs=(orc.SbsHeader(h.brick_size, h.brick_pad, h.bytes_per_value, h.aux_data), nodes, values),
                     pairs=pairs, intersect=2, render_mode=8, closest_hit=True)


def _rays():
    views = scenes.proposal_views(16, 1024, seed=8)
    return [(views[int(v)], int(p), np.float32(t), int(k))
            for v, p, t, k in zip(GOLD["view"], GOLD["pixel"], GOLD["t"], GOLD["prim"])]


def test_oracle_walks_grazing_rays_to_their_end():
    h, nodes, values = _fixture()
    osc = _oracle(h, nodes, values)
    for (w, hh, wv, pj), pix, t, k in _rays():
        o, cnt = osc.render_pixels(w, hh, lrt.inverse4x4(pj), lrt.inverse4x4(wv), np.array([pix], np.uint32), threads=1)
        assert o["primId"][0] == k and o["t"][0] == t
        # more voxel steps on the ray than 8 * brick_size + 16 (the old bound of one brick)
        assert cnt.n_vox > 8 * h.brick_size + 16


@pytest.mark.gpu
def test_engine_walks_grazing_rays_like_the_oracle():
    """The 40 bricks of the fixture, and the full 1024^3 scene (built on the GPU)."""
    full = lrt.sbs_from_sdf(scenes.union_sdf(), 7, 8, gpu=0)
    for scene, ids in ((_fixture(), None), (full, GOLD["full_index"])):
        h, nodes, values = scene
        s = lrt.Scene(0)
        try:
            s.add_instance(s.add_sbs(h, nodes, values))
            s.commit_scene()
            s.set_preset(render_mode=lrt.RENDER_MODE_NORMAL, sdf_node_intersect=lrt.INTERSECT_NEWTON)
            for view, pix, t, k in _rays():
                got = s.render_host([view], hits=True)["hits"][pix]
                assert got["primId"] == (k if ids is None else ids[k])
                assert np.float32(got["t"]).view(np.uint32) == t.view(np.uint32)
        finally:
            s.close()
