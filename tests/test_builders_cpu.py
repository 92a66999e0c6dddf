"""CPU: the engine's scene construction and BVH builder against the oracle.

The SBS/SVS builders restate utils/sparse_octree_builder.cpp (frame octree,
border-brick test, DX quantisation); product and oracle must agree bit for bit.
"""
import numpy as np
import pytest

from litert_gb300 import lrt, scenes
from oracle import oracle as orc

SPHERE = scenes.SPHERE_SDF


@pytest.mark.parametrize("depth,bs,pad,bpv", [(4, 4, 0, 4), (6, 4, 0, 4), (5, 2, 1, 2), (4, 1, 0, 1), (3, 8, 0, 4)])
def test_sbs_sphere_bit_exact(depth, bs, pad, bpv):
    h, n, v = lrt.sbs_from_sdf(lrt.Sdf(**SPHERE), depth, bs, pad, bpv)
    h2, n2, v2 = orc.build_sbs(SPHERE["spheres"], None, 0.0, depth, bs, pad, bpv)
    assert n.shape[0] > 0
    assert np.array_equal(n, n2)
    assert np.array_equal(v, v2)
    assert (h.brick_size, h.brick_pad, h.bytes_per_value) == (bs, pad, bpv)


def test_sbs_union_bit_exact():
    p = scenes.union_params()
    h, n, v = lrt.sbs_from_sdf(lrt.Sdf(**p), 5, 4)
    h2, n2, v2 = orc.build_sbs(p["spheres"], p["boxes"], p["k"], 5, 4)
    assert np.array_equal(n, n2) and np.array_equal(v, v2)


def test_sbs_thread_count_invariant():
    p = scenes.union_params()
    a = lrt.sbs_from_sdf(lrt.Sdf(**p), 5, 2, threads=1)
    b = lrt.sbs_from_sdf(lrt.Sdf(**p), 5, 2, threads=7)
    assert np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2])


@pytest.mark.parametrize("depth", [4, 6])
def test_svs_bit_exact(depth):
    n = lrt.svs_from_sdf(lrt.Sdf(**SPHERE), depth)
    n2 = orc.build_svs(SPHERE["spheres"], None, 0.0, depth)
    assert n.shape[0] > 0 and np.array_equal(n, n2)


def test_border_brick_property():
    """Every kept brick straddles or hugs the surface: min <= 0 < max + d_max (is_border_node)."""
    h, n, v = lrt.sbs_from_sdf(lrt.Sdf(**SPHERE), 4, 4)
    lod = n[:, 1] & 0xFFFF
    d_max = 2 * np.sqrt(3.0) / lod
    vals = v.reshape(n.shape[0], -1).astype(np.float64)
    dec = -d_max[:, None] + (2 * d_max[:, None] / 4294967295.0) * vals
    assert (dec.min(1) <= 1e-6).all()
    assert (dec.max(1) > -d_max - 1e-6).all()


def _check_bvh2(pairs_bytes, n_prims, boxes, prims_per_leaf, sc=None):
    P = np.frombuffer(pairs_bytes.tobytes(), lrt.BVH_PAIR_DTYPE)
    seen = []
    stack = [0]
    while stack:
        i = stack.pop()
        for side in ("l", "r"):
            lo, hi, ref = P[i][side + "min"], P[i][side + "max"], int(P[i][side + "left"])
            if ref & 0x80000000:
                payload = ref & 0x00FFFFFF
                if prims_per_leaf == 1:
                    seen.append(payload)
                    assert (lo <= boxes[payload, :3]).all() and (hi >= boxes[payload, 3:]).all()
                else:
                    st = int(sc[payload])
                    seen.extend(range(st & 0xFFFFFF, (st & 0xFFFFFF) + ((st >> 24) & 0x7F)))
            else:
                assert ref < P.size
                for s2 in ("l", "r"):   # child boxes are enclosed by this box
                    assert (lo <= P[ref][s2 + "min"]).all() and (hi >= P[ref][s2 + "max"]).all()
                stack.append(ref)
    return seen


def test_bvh2_boxes_cover_every_leaf_once():
    h, n, v = lrt.sbs_from_sdf(lrt.Sdf(**SPHERE), 5, 4)
    boxes = orc.node_boxes(n)
    pairs, sc, order = lrt.build_bvh2(boxes, 1)
    seen = _check_bvh2(pairs, n.shape[0], boxes, 1)
    assert sorted(seen) == list(range(n.shape[0]))


def test_bvh2_triangles_cover_every_triangle_once():
    verts, faces = scenes.displaced_icosphere(subdiv=3)
    tri = verts[faces]
    boxes = np.concatenate([tri.min(1), tri.max(1)], 1)
    pairs, sc, order = lrt.build_bvh2(boxes, 2)
    seen = _check_bvh2(pairs, faces.shape[0], boxes, 2, sc)
    assert sorted(seen) == list(range(faces.shape[0]))
    assert sorted(order.tolist()) == list(range(faces.shape[0]))


def test_single_box_bvh():
    boxes = np.array([[0, 0, 0, 1, 1, 1]], np.float32)
    pairs, sc, order = lrt.build_bvh2(boxes, 1)
    P = np.frombuffer(pairs.tobytes(), lrt.BVH_PAIR_DTYPE)
    assert P.size == 1 and int(P[0]["lleft"]) & 0x80000000


def test_invalid_builder_args():
    with pytest.raises(lrt.LrtError):
        lrt.sbs_from_sdf(lrt.Sdf(**SPHERE), 4, 0)        # brick size 0
    with pytest.raises(lrt.LrtError):
        lrt.sbs_from_sdf(lrt.Sdf(**SPHERE), 4, 4, bytes_per_value=3)
