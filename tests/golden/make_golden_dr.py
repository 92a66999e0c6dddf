"""Generate tests/golden/ref_dr_payload.npz from the reference's own DR code.

Runs where the reference tree is present: builds oracle/_ref (the reference's
BVH/BVH2Common.cpp and diff_render/BVH2DR.cpp compiled in place,
oracle/build_ref.py) and records, for a small seeded indexed SBS grid, the
scene, the BVH2, a selection of rays and the RayQuery_NearestHitWithGrad
records (hit + RayDiffPayload) the reference returns for the ray-flag sets the
differentiable render uses.  tests/test_oracle_dr_pin_cpu.py checks the CPU
oracle against these records bit for bit.

    python tests/golden/make_golden_dr.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from litert_gb300 import lrt, scenes  # noqa: E402
from oracle import oracle as orc  # noqa: E402
from oracle import oracle_dr as od  # noqa: E402
from oracle import ref  # noqa: E402

OUT = os.path.join(HERE, "ref_dr_payload.npz")
FLAG_SETS = (1 | 2 | 4, 8, 16)


def scene():
    up = scenes.union_params()
    hdr, nodes, values, params = od.grid_sbs(6, 4, spheres=up["spheres"], boxes=up["boxes"], k=up["k"])
    rng = np.random.default_rng(11)
    nd = 25 ** 3
    params = params.copy()
    params[:nd] += rng.normal(0, 0.005, nd).astype(np.float32)
    params[nd:] = rng.uniform(0, 1, params.size - nd).astype(np.float32)
    return hdr, nodes, values, params


def rays():
    P, D = [], []
    for (w, h, wv, pj) in scenes.union_views(n_views=2, lo=64, hi=80):
        pos, dr = orc.eye_rays(w, h, lrt.inverse4x4(pj), lrt.inverse4x4(wv), np.arange(w * h, dtype=np.uint32), 0.3, 0.7)
        P.append(pos)
        D.append(dr)
    return np.concatenate(P), np.concatenate(D)


def main():
    hdr, nodes, values, params = scene()
    sc = od.DrScene(hdr, nodes, values, params.size)
    rs = ref.RefScene("sbs", (hdr, nodes, values, params), sc.pairs, (17, 2, 0, 0, 0, 1, 1))
    P, D = rays()
    hit = rs.dr_query(1 | 2 | 4, P, D)["hit"]["primId"] != 0xFFFFFFFF
    border = rs.dr_query(8, P, D)["missed_hit"]["sdf"] < 1e-3
    rng = np.random.default_rng(12)
    sel = np.concatenate([rng.choice(np.nonzero(hit)[0], 300, replace=False), np.nonzero(border)[0][:80],
                          rng.choice(np.nonzero(~hit & ~border)[0], 60, replace=False)])
    out = dict(hdr=np.array([hdr.brick_size, hdr.brick_pad, hdr.bytes_per_value, hdr.aux_data], np.uint32),
               nodes=nodes, values=values, params=params, pairs=sc.pairs, pos=P[sel], dir=D[sel])
    for f in FLAG_SETS:
        out[f"rec_{f}"] = rs.dr_query(f, P[sel], D[sel])
    np.savez_compressed(OUT, **out)
    print(OUT, os.path.getsize(OUT), "bytes", len(sel), "rays")


if __name__ == "__main__":
    main()
