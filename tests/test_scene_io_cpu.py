"""CPU: SBS / SVS files in the reference's binary layout (save_sdf_SBS /
load_sdf_SBS / save_sdf_SVS / load_sdf_SVS, sdfScene/sdf_scene.cpp:121-175).

Round trips through our writer and reader; the byte layout written field by
field against the reference's description (header, u32 count, nodes, u32
count, values); short and foreign files rejected.  Where the reference tree is
present, its own fixtures saves/test_10_sbs.bin and saves/test_10_svs.bin (used
by tests/tests.cpp:1311-1312) load through our reader, and the oracle and the
reference's BVHRT, compiled in place, return the same hits on them."""
import os
import struct

import numpy as np
import pytest

from litert_gb300 import lrt, scenes
from oracle import oracle as orc

from oracle.build_ref import REF as REF_TREE   # the one place that locates the reference tree


def _sbs():
    return lrt.sbs_from_sdf(lrt.Sdf(**scenes.SPHERE_SDF), 4, 4, 1, 2)


def test_sbs_round_trip_and_layout(tmp_path):
    h, n, v = _sbs()
    p = tmp_path / "a.bin"
    lrt.save_sbs(p, h, n, v)
    raw = p.read_bytes()
    assert len(raw) == 16 + 4 + n.size * 4 + 4 + v.size * 4
    assert struct.unpack_from("<4I", raw, 0) == (h.brick_size, h.brick_pad, h.bytes_per_value, h.aux_data)
    assert struct.unpack_from("<I", raw, 16)[0] == n.shape[0]
    assert np.array_equal(np.frombuffer(raw, np.uint32, n.size, 20).reshape(-1, 4), n)
    assert struct.unpack_from("<I", raw, 20 + n.size * 4)[0] == v.size
    h2, n2, v2 = lrt.load_sbs(p)
    assert (h2.brick_size, h2.brick_pad, h2.bytes_per_value, h2.aux_data) == \
           (h.brick_size, h.brick_pad, h.bytes_per_value, h.aux_data)
    assert np.array_equal(n2, n) and np.array_equal(v2, v)


def test_svs_round_trip_and_layout(tmp_path):
    n = lrt.svs_from_sdf(lrt.Sdf(**scenes.SPHERE_SDF), 5)
    p = tmp_path / "a.bin"
    lrt.save_svs(p, n)
    raw = p.read_bytes()
    assert len(raw) == 4 + n.size * 4 and struct.unpack_from("<I", raw, 0)[0] == n.shape[0]
    assert np.array_equal(lrt.load_svs(p), n)


def test_empty_sets(tmp_path):
    h, _, _ = _sbs()
    p = tmp_path / "e.bin"
    lrt.save_sbs(p, h, np.zeros((0, 4), np.uint32), np.zeros(0, np.uint32))
    _, n, v = lrt.load_sbs(p)
    assert n.shape == (0, 4) and v.size == 0
    lrt.save_svs(p, np.zeros((0, 4), np.uint32))
    assert lrt.load_svs(p).shape == (0, 4)


def test_short_and_foreign_files_rejected(tmp_path):
    h, n, v = _sbs()
    p = tmp_path / "a.bin"
    lrt.save_sbs(p, h, n, v)
    raw = p.read_bytes()
    for cut in (0, 10, 19, 20 + 16, len(raw) - 4, len(raw) - 1):
        q = tmp_path / f"cut{cut}.bin"
        q.write_bytes(raw[:cut])
        with pytest.raises(lrt.LrtError):
            lrt.load_sbs(q)
    q = tmp_path / "huge.bin"                       # a node count far beyond the file
    q.write_bytes(raw[:16] + struct.pack("<I", 0x7FFFFFFF) + raw[20:])
    with pytest.raises(lrt.LrtError):
        lrt.load_sbs(q)
    q.write_bytes(struct.pack("<I", 1000) + b"\0" * 32)
    with pytest.raises(lrt.LrtError):
        lrt.load_svs(q)
    with pytest.raises(lrt.LrtError):
        lrt.load_sbs(tmp_path / "missing.bin")


live = pytest.mark.skipif(not os.path.exists(os.path.join(REF_TREE, "saves", "test_10_sbs.bin")) or
                          not __import__("oracle.ref", fromlist=["x"]).available(),
                          reason="reference fixtures not present")


def _bits(a):
    f = np.ascontiguousarray(a).view(np.float32).copy()
    b = f.view(np.uint32).copy()
    b[np.isnan(f)] = 0x7FC00000
    return b.reshape(a.size, -1)


@live
def test_reference_sbs_fixture_loads_and_renders_like_the_reference():
    from oracle import ref
    h, n, v = lrt.load_sbs(os.path.join(REF_TREE, "saves", "test_10_sbs.bin"))
    assert (h.brick_size, h.brick_pad, h.bytes_per_value) == (1, 0, 1) and n.shape[0] == 49487 and v.size == 98974
    pairs = lrt.build_bvh2(orc.node_boxes(n), 1)
    oh = orc.SbsHeader(h.brick_size, h.brick_pad, h.bytes_per_value, h.aux_data)
    w = hh = 128   # the fixture's test renders from (0, 0, 3) towards the origin
    pj = lrt.perspective(60.0, 1.0, 0.01, 100.0)
    wv = lrt.look_at([0, 0, 3], [0, 0, 0], [0, 1, 0])
    pos, dr = ref.eye_rays(w, hh, lrt.inverse4x4(pj), lrt.inverse4x4(wv), np.arange(w * hh, dtype=np.uint32))
    a = ref.RefScene("sbs", (oh, n, v), pairs[0], (8, 2, 0, 0, 0, 1, 1)).query(pos, dr)
    b = orc.Scene("sbs", sbs=(oh, n, v), pairs=pairs, intersect=2, render_mode=8, closest_hit=False).query_rays(pos, dr)
    assert (a["primId"] != lrt.MISS).sum() > 1000
    assert np.array_equal(_bits(a), _bits(b))


@live
def test_reference_svs_fixture_loads_and_renders_like_the_reference():
    from oracle import ref
    n = lrt.load_svs(os.path.join(REF_TREE, "saves", "test_10_svs.bin"))
    assert n.shape[0] == 49487
    pairs = lrt.build_bvh2(orc.node_boxes(n), 1)   # the SVS node position encoding is the SBS one
    w = hh = 128
    pj = lrt.perspective(60.0, 1.0, 0.01, 100.0)
    wv = lrt.look_at([0, 0, 3], [0, 0, 0], [0, 1, 0])
    pos, dr = ref.eye_rays(w, hh, lrt.inverse4x4(pj), lrt.inverse4x4(wv), np.arange(w * hh, dtype=np.uint32))
    a = ref.RefScene("svs", n, pairs[0], (8, 2, 0, 0, 0, 1, 1)).query(pos, dr)
    b = orc.Scene("svs", svs=n, pairs=pairs, intersect=2, render_mode=8, closest_hit=False).query_rays(pos, dr)
    assert (a["primId"] != lrt.MISS).sum() > 1000
    assert np.array_equal(_bits(a), _bits(b))
