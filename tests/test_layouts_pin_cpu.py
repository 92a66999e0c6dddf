"""CPU: the coloured (DX_RGB8) and textured (DX_UV16) brick layouts in the oracle
against the reference's own BVHRT::RayQuery_NearestHit (BVH/BVH2Common.cpp
compiled in place), through the committed records tests/golden/ref_layouts.npz
(tests/golden/make_golden_layouts.py): every hit record -- distance, brick,
colour or texture coordinates (coords[0..1]) and normal -- bit for bit."""
import os

import numpy as np
import pytest

from oracle import oracle as orc

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden", "ref_layouts.npz")
RAYS = os.path.join(HERE, "golden", "ref_rayquery.npz")
CASES = ("rgb8_q4", "rgb8_q1pad", "uv16_q2")


def _bits(a):
    f = np.ascontiguousarray(a).view(np.float32).copy()
    b = f.view(np.uint32).copy()
    b[np.isnan(f)] = 0x7FC00000
    return b.reshape(a.size, -1)


@pytest.mark.parametrize("case", CASES)
def test_layout_hits_match_reference(case):
    g = np.load(GOLD)
    r = np.load(RAYS)
    hdr = [int(x) for x in g[case + "_hdr"]]
    oh = orc.SbsHeader(*hdr)
    sc = orc.Scene("sbs", sbs=(oh, g[case + "_nodes"], g[case + "_values"]), pairs=(g[case + "_pairs"], None, None),
                   intersect=2, render_mode=8, closest_hit=False)
    got = sc.query_rays(r["rays_pos"], r["rays_dir"])
    want = g[case + "_hits"]
    assert (want["primId"] != 0xFFFFFFFF).sum() > 300
    assert np.array_equal(_bits(got), _bits(want))


@pytest.mark.parametrize("normal_mode", [0, 2])
def test_smoothed_normals_match_reference(normal_mode):
    """NORMAL_MODE_SDF_SMOOTHED (BVH/BVH2Common.cpp:838-905) on a create_grid_sbs set
    with neighbour ids: the smoothed normals bit for bit, and the plain ones for contrast."""
    g = np.load(GOLD)
    r = np.load(RAYS)
    oh = orc.SbsHeader(*[int(x) for x in g["smooth_hdr"]])
    sc = orc.Scene("sbs", sbs=(oh, g["smooth_nodes"], g["smooth_values"], g["smooth_values_f"]),
                   pairs=(g["smooth_pairs"], None, None), intersect=2, render_mode=8, closest_hit=False,
                   normal_mode=normal_mode)
    got = sc.query_rays(r["rays_pos"], r["rays_dir"])
    want = g[f"smooth_hits_n{normal_mode}"]
    assert (want["primId"] != 0xFFFFFFFF).sum() > 300
    assert np.array_equal(_bits(got), _bits(want))


def test_smoothing_changes_the_normals():
    g = np.load(GOLD)
    a, b = g["smooth_hits_n0"], g["smooth_hits_n2"]
    hit = a["primId"] != 0xFFFFFFFF
    assert np.array_equal(a["t"], b["t"])
    assert (a["coords"][hit, 2] != b["coords"][hit, 2]).mean() > 0.5
