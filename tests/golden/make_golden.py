"""Generate tests/golden/ref_rayquery.npz from the reference's own code.

Runs where the reference tree is present: builds oracle/_ref (the reference's
BVH/BVH2Common.cpp compiled in place, oracle/build_ref.py) and records, for
small seeded scenes, the scene data, the BVH2 used, the rays and the hits
returned by the reference's BVHRT::RayQuery_NearestHit for every finder mode,
plus the reference's eye rays (render_common.h).  tests/test_oracle_pin_cpu.py
checks the CPU oracle against these records bit for bit.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from litert_gb300 import lrt, scenes  # noqa: E402
from oracle import oracle as orc  # noqa: E402
from oracle import ref  # noqa: E402

OUT = os.path.join(HERE, "ref_rayquery.npz")
MODES = (2, 0, 1, 3, 4)   # NEWTON, ST, ANALYTIC, BBOX, IT


def rays(seed=1, n=3000):
    rng = np.random.default_rng(seed)
    p = np.zeros((n, 4), np.float32)
    p[:, :3] = rng.uniform(-2, 2, (n, 3))
    p[:, 3] = rng.choice([0.0, 0.3], n)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    dd = np.zeros((n, 4), np.float32)
    dd[:, :3] = d
    dd[:, 3] = 1e9
    return p, dd


def main():
    out = {}
    w, h, wv, pj = scenes.sphere_view(48, 40)
    pi, wi = lrt.inverse4x4(pj), lrt.inverse4x4(wv)
    pix = np.arange(w * h, dtype=np.uint32)
    ep, ed = ref.eye_rays(w, h, pi, wi, pix)
    out.update(eye_w=w, eye_h=h, eye_proj_inv=pi, eye_wv_inv=wi, eye_pos=ep, eye_dir=ed)
    rp, rd = rays()
    P = np.concatenate([ep, rp])
    D = np.concatenate([ed, rd])
    out.update(rays_pos=P, rays_dir=D)

    cases = {
        "sbs_sphere": ("sbs", scenes.SPHERE_SDF, 3, 4, 0, 4),
        "sbs_union": ("sbs", scenes.union_params(), 4, 2, 0, 4),
        "sbs_union_q8pad": ("sbs", scenes.union_params(), 3, 4, 1, 1),
    }
    for name, (_, params, depth, bs, pad, bpv) in cases.items():
        hd, n, v = lrt.sbs_from_sdf(lrt.Sdf(**params), depth, bs, pad, bpv)
        pairs, sc, order = lrt.build_bvh2(orc.node_boxes(n), 1)
        oh = orc.SbsHeader(hd.brick_size, hd.brick_pad, hd.bytes_per_value, hd.aux_data)
        out[name + "_hdr"] = np.array([hd.brick_size, hd.brick_pad, hd.bytes_per_value, hd.aux_data], np.uint32)
        out[name + "_nodes"], out[name + "_values"], out[name + "_pairs"] = n, v, pairs
        for m in MODES:
            rs = ref.RefScene("sbs", (oh, n, v), pairs, (8, m, 0, 0, 0, 1, 1))
            out[f"{name}_hits_m{m}"] = rs.query(P, D)

    n = lrt.svs_from_sdf(lrt.Sdf(**scenes.SPHERE_SDF), 4)
    pairs, sc, order = lrt.build_bvh2(orc.node_boxes(n), 1)
    out["svs_sphere_nodes"], out["svs_sphere_pairs"] = n, pairs
    for m in MODES:
        rs = ref.RefScene("svs", n, pairs, (8, m, 0, 0, 0, 1, 1))
        out[f"svs_sphere_hits_m{m}"] = rs.query(P, D)

    verts, faces = scenes.displaced_icosphere(subdiv=2)
    tri = verts[faces]
    pairs, sc, order = lrt.build_bvh2(np.concatenate([tri.min(1), tri.max(1)], 1), 2)
    v4 = np.ones((verts.shape[0], 4), np.float32)
    v4[:, :3] = verts
    rs = ref.RefScene("tri", (v4, faces, order, sc), pairs, (8, 2, 0, 0, 0, 1, 1))
    out.update(tri_verts=verts, tri_faces=faces, tri_pairs=pairs, tri_sc=sc, tri_order=order,
               tri_hits=rs.query(P, D))
    np.savez_compressed(OUT, **out)
    print(OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
