"""Generates tests/golden/walk_bound_grazing.npz: the bricks that two grazing rays
of the proposal benchmark's held-out views cross in the 1024^3 smooth-union scene
(depth 7, 8-voxel bricks), for tests/test_walk_bound.py.

The rays take more voxel steps in one brick than 8 * brick_size + 16 (their
positions keep rounding back into voxels they have left, so a step advances t by
the bare +1e-6).  Every brick whose box a ray crosses is kept, so the closest hit
over the kept bricks is the full scene's.  Stored: the SBS header, the kept nodes
(data offsets renumbered) and their values, each ray's view and pixel, and the
closest hit of a walk without a step bound (t and the kept-brick index), taken
from the oracle built with its bound lifted (the bound is the only difference).

Run from the repository root: python tests/golden/make_golden_walk_bound.py
(takes about a minute: the host builder and two oracle builds).
"""
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from litert_gb300 import lrt, scenes  # noqa: E402
from oracle import oracle as orc  # noqa: E402

RAYS = [(11, 371353), (12, 813364)]   # (view, pixel) of scenes.proposal_views(16, 1024, seed=8)


def unbounded_oracle(tmp):
    """The oracle's sources with the walk's step bound lifted, built into tmp."""
    src = open(os.path.join(ROOT, "oracle", "lrt_oracle.c")).read()
    src, n = re.subn(r"const uint32_t max_steps = orc_walk_step_bound\([^;]*\);", "const uint32_t max_steps = 1u << 30;",
                     src)
    assert n == 1
    open(os.path.join(tmp, "lrt_oracle.c"), "w").write(src)
    lib = os.path.join(tmp, "liblrt_oracle.so")
    subprocess.check_call(["gcc", "-O2", "-std=c11", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
                           "-I" + os.path.join(ROOT, "oracle"), "-o", lib, os.path.join(tmp, "lrt_oracle.c"),
                           os.path.join(ROOT, "oracle", "lrt_oracle_build.c"),
                           os.path.join(ROOT, "oracle", "lrt_oracle_dr.c"), "-lm"])
    return lib


def crossed(boxes, pos, d):
    inv = np.float64(1.0) / np.where(d == 0, 1e-30, d)
    t0 = (boxes[:, :3] - pos) * inv
    t1 = (boxes[:, 3:] - pos) * inv
    tn = np.minimum(t0, t1).max(1)
    tf = np.maximum(t0, t1).min(1)
    return np.nonzero((tn <= tf) & (tf >= 0))[0]


def main():
    h, nodes, values = lrt.sbs_from_sdf(scenes.union_sdf(), 7, 8)
    views = scenes.proposal_views(16, 1024, seed=8)
    boxes = orc.node_boxes(nodes).astype(np.float64)
    keep = set()
    for vi, pix in RAYS:
        w, hh, wv, pj = views[vi]
        p, d = orc.eye_rays(w, hh, lrt.inverse4x4(pj), lrt.inverse4x4(wv), np.array([pix], np.uint32))
        keep.update(crossed(boxes, p[0, :3].astype(np.float64), d[0, :3].astype(np.float64)).tolist())
    keep = np.array(sorted(keep), np.int64)
    v3 = (h.brick_size + 2 * h.brick_pad + 1) ** 3
    sub_nodes = nodes[keep].copy()
    sub_values = np.concatenate([values[int(nodes[k, 2]):int(nodes[k, 2]) + v3] for k in keep])
    sub_nodes[:, 2] = np.arange(len(keep), dtype=np.uint32) * v3
    with tempfile.TemporaryDirectory() as tmp:
        orc.LIB_PATH = unbounded_oracle(tmp)
        orc._lib = None   # load the unbounded build from here on
        pairs = lrt.build_bvh2(orc.node_boxes(sub_nodes), 1)
        osc = orc.Scene("sbs", sbs=(orc.SbsHeader(h.brick_size, h.brick_pad, h.bytes_per_value, h.aux_data), sub_nodes,
                                    sub_values), pairs=pairs, intersect=2, render_mode=8, closest_hit=True)
        ts, prims = [], []
        for vi, pix in RAYS:
            w, hh, wv, pj = views[vi]
            o, _ = osc.render_pixels(w, hh, lrt.inverse4x4(pj), lrt.inverse4x4(wv), np.array([pix], np.uint32),
                                     threads=1)
            ts.append(o["t"][0])
            prims.append(o["primId"][0])
    out = os.path.join(ROOT, "tests", "golden", "walk_bound_grazing.npz")
    np.savez_compressed(out, header=np.array([h.brick_size, h.brick_pad, h.bytes_per_value, h.aux_data], np.uint32),
                        nodes=sub_nodes, values=sub_values, full_index=keep.astype(np.uint32),
                        view=np.array([v for v, _ in RAYS], np.uint32), pixel=np.array([p for _, p in RAYS], np.uint32),
                        t=np.array(ts, np.float32), prim=np.array(prims, np.uint32))
    print(out, len(keep), "bricks", ts, prims, keep[np.array(prims)])


if __name__ == "__main__":
    main()
