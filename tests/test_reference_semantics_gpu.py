"""GPU parity against the reference's own semantics at the benchmark sizes.

* Triangle mesh at full size: the 327,680-triangle displaced icosphere rendered at
  1920x1080 from the seeded camera, compared on every pixel with the oracle (IntersectAllTrianglesInLeaf, BVH/BVH2Common.cpp:2776-2840;
  triangles have no first-hit early-out, so the reference returns the closest hit
  too).  The bar is the forward tolerance: hit mask identical apart from < 0.01 %
  of the pixels, depth within 1e-4 of the scene extent (2), normals within 1e-3;
  the rate at which a ray meets two triangles at exactly the same distance
  (shared-edge ties, where primId may name either neighbour) is measured.
* Closest hit against the reference's first hit: BVH2TraverseF32 stops at the
  first SDF leaf that reports a hit (BVH/BVH2Common.cpp:3402-3405, 3478), the
  default kernels return the closest one.  On the small sphere configuration (all
  65,536 pixels) the two agree within the tolerance (measured: no difference).
  On the 16-view 1024^3 headline (all 33.6 M pixels) they do not: about 0.4 % of
  the pixels hit a farther brick first, where sibling boxes of the BVH2 overlap --
  a property of the reference's early-out on a given tree, not of the arithmetic.
  The "first_hit" tuning reproduces the reference's result on the same tree bit
  for bit on every pixel (NaN normals of zero gradients compared as NaN), and the count of closest-vs-first differences is held to
  its measured size.  The oracle runs on all host cores.
"""
import os

import numpy as np
import pytest

from litert_gb300 import lrt, scenes
from oracle import oracle as orc

from _util import canon_bits

pytestmark = pytest.mark.gpu

EXTENT = 2.0            # the [-1, 1]^3 scene cube
DEPTH_TOL = 1e-4 * EXTENT
MASK_FRAC = 1e-4        # 0.01 % of the pixels


THREADS = os.cpu_count() or 1


def _all_pixels(views):
    out, off = [], 0
    for vi, (w, h, _, _) in enumerate(views):
        out.append((vi, off, np.arange(w * h, dtype=np.uint32)))
        off += w * h
    return out


def _decode(nx, ny):
    """Octahedral decode of the stored normal (the inverse of encode_normal)."""
    nx = np.asarray(nx, np.float64)
    ny = np.asarray(ny, np.float64)
    z = 1.0 - np.abs(nx) - np.abs(ny)
    x = np.where(z >= 0, nx, (1.0 - np.abs(ny)) * np.where(nx >= 0, 1.0, -1.0))
    y = np.where(z >= 0, ny, (1.0 - np.abs(nx)) * np.where(ny >= 0, 1.0, -1.0))
    v = np.stack([x, y, z], 1)
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def _tolerance_report(g, o):
    """g: engine HIT16 records, o: oracle CRT_Hit records of the same pixels."""
    mg, mo = g["primId"] != lrt.MISS, o["primId"] != lrt.MISS
    both = mg & mo
    dt = np.abs(g["t"][both].astype(np.float64) - o["t"][both].astype(np.float64))
    return dict(n=int(g.size), hits=int(mo.sum()), mask=int((mg != mo).sum()), depth=int((dt > DEPTH_TOL).sum()),
                max_dt=float(dt.max()) if dt.size else 0.0, both=both)


def test_mesh_full_size_against_oracle():
    verts, faces = scenes.displaced_icosphere(subdiv=7)
    assert faces.shape[0] == 327_680
    view = scenes.mesh_view()
    w, h, wv, pj = view
    assert (w, h) == (1920, 1080)
    s = lrt.Scene(0)
    s.add_instance(s.add_triangles(verts, faces))
    s.commit_scene()
    s.set_preset(render_mode=lrt.RENDER_MODE_NORMAL)
    g_all = s.render_host([view], hits=True)["hits"]
    s.close()
    osc = orc.Scene("mesh", mesh=(verts, faces), render_mode=lrt.RENDER_MODE_NORMAL)
    pix = np.arange(w * h, dtype=np.uint32)
    o, _ = osc.render_pixels(w, h, lrt.inverse4x4(pj), lrt.inverse4x4(wv), pix, threads=THREADS)
    g = g_all
    r = _tolerance_report(g, o)
    assert r["n"] == w * h and r["hits"] > 500_000, r
    assert r["mask"] <= MASK_FRAC * r["n"], r
    assert r["depth"] == 0, r
    both = r["both"]
    same = both & (g["primId"] == o["primId"])
    ties = both & ~same
    # a tie is a ray that meets two triangles at one distance: t is identical
    assert np.array_equal(g["t"][ties], o["t"][ties])
    tie_rate = ties.sum() / max(1, both.sum())
    assert tie_rate <= 1e-3, tie_rate
    ng = _decode(g["nx"][same], g["ny"][same])
    no = _decode(o["coords"][same, 2], o["coords"][same, 3])
    assert np.abs(ng - no).max() <= 1e-3
    # the kernel is the uncontracted one: depths are bit-identical
    assert np.array_equal(g["t"][both].view(np.uint32), o["t"][both].view(np.uint32))
    print(f"mesh 1920x1080: {r['n']} rays, {r['hits']} hits, mask diffs {r['mask']}, "
          f"shared-edge ties {int(ties.sum())} ({tie_rate:.2e} of hits)")


def _first_hit_counts(s, osc_first, views, sample, fma):
    s.set_tuning("fma", fma)
    g_all = s.render_host(views, hits=True)["hits"]
    n = mask = depth = hits = 0
    max_dt = 0.0
    for vi, off, pix in sample:
        w, hh, wv, pj = views[vi]
        o, _ = osc_first.render_pixels(w, hh, lrt.inverse4x4(pj), lrt.inverse4x4(wv), pix, threads=THREADS)
        r = _tolerance_report(g_all[off + pix.astype(np.int64)], o)
        n += r["n"]
        hits += r["hits"]
        mask += r["mask"]
        depth += r["depth"]
        max_dt = max(max_dt, r["max_dt"])
    return dict(n=n, hits=hits, mask=mask, depth=depth, max_dt=max_dt)


@pytest.mark.parametrize("fma", [0, 1])
def test_closest_vs_first_hit_sphere(fma):
    h, n, v = lrt.sbs_from_sdf(scenes.sphere_sdf(), 4, 4)
    view = scenes.sphere_view(256, 256)
    s = lrt.Scene(0)
    s.add_instance(s.add_sbs(h, n, v))
    s.commit_scene()
    s.set_preset(render_mode=lrt.RENDER_MODE_NORMAL, sdf_node_intersect=lrt.INTERSECT_NEWTON)
    osc = orc.Scene("sbs", sbs=(orc.SbsHeader(h.brick_size, h.brick_pad, h.bytes_per_value, h.aux_data), n, v),
                    pairs=(s.bvh2(), None, None), intersect=lrt.INTERSECT_NEWTON,
                    render_mode=lrt.RENDER_MODE_NORMAL, closest_hit=False)
    sample = [(0, 0, np.arange(256 * 256, dtype=np.uint32))]
    r = _first_hit_counts(s, osc, [view], sample, fma)
    s.close()
    print(f"sphere 256^2 fma={fma}: {r}")
    assert r["n"] == 65536 and r["hits"] > 6000
    assert r["mask"] + r["depth"] <= MASK_FRAC * r["n"], r


@pytest.fixture(scope="module")
def headline():
    h, nodes, values = lrt.sbs_from_sdf(scenes.union_sdf(), 7, 8, gpu=0)
    s = lrt.Scene(0)
    s.add_instance(s.add_sbs(h, nodes, values))
    s.commit_scene()
    s.set_preset(render_mode=lrt.RENDER_MODE_NORMAL, sdf_node_intersect=lrt.INTERSECT_NEWTON)
    views = scenes.union_views()
    osc = orc.Scene("sbs", sbs=(orc.SbsHeader(h.brick_size, h.brick_pad, h.bytes_per_value, h.aux_data), nodes,
                                values), pairs=(s.bvh2(), None, None), intersect=lrt.INTERSECT_NEWTON,
                    render_mode=lrt.RENDER_MODE_NORMAL, closest_hit=False)
    yield s, osc, views
    s.close()


@pytest.mark.parametrize("fma", [0, 1])
def test_closest_vs_first_hit_headline(headline, fma):
    s, osc, views = headline
    r = _first_hit_counts(s, osc, views, _all_pixels(views), fma)
    print(f"headline 16 views fma={fma}: {r}")
    assert r["n"] == sum(w * h for w, h, _, _ in views) and r["hits"] > 5_000_000
    assert r["mask"] <= MASK_FRAC * r["n"], r
    # first hits in a farther brick behind overlapping boxes (measured: 212 of a 48,000-pixel sample)
    assert r["depth"] <= 0.01 * r["n"], r


def test_first_hit_mode_reproduces_reference_on_headline(headline):
    s, osc, views = headline
    s.set_tuning("fma", 0)
    s.set_tuning("first_hit", 1)
    try:
        g_all = s.render_host(views, hits=True)["hits"]
    finally:
        s.set_tuning("first_hit", 0)
    n = 0
    for vi, off, pix in _all_pixels(views):
        w, hh, wv, pj = views[vi]
        o, _ = osc.render_pixels(w, hh, lrt.inverse4x4(pj), lrt.inverse4x4(wv), pix, threads=THREADS)
        g = g_all[off + pix.astype(np.int64)]
        assert np.array_equal(g["primId"], o["primId"])
        hit = o["primId"] != lrt.MISS
        assert np.array_equal(g["t"][hit].view(np.uint32), o["t"][hit].view(np.uint32))
        # bit for bit; a zero gradient's normal is NaN on both sides, with the payload of
        # each machine (measured: 63 of 9.9 M hits)
        assert np.array_equal(canon_bits(g["nx"][hit]), canon_bits(o["coords"][hit, 2]))
        assert np.array_equal(canon_bits(g["ny"][hit]), canon_bits(o["coords"][hit, 3]))
        n += pix.size
    assert n == sum(w * h for w, h, _, _ in views)
