"""Generate tests/golden/ref_layouts.npz from the reference's own code: the
coloured (DX_RGB8) and textured (DX_UV16) brick layouts, and smoothed normals
(NORMAL_MODE_SDF_SMOOTHED) on the neighbour layout (ID32F_IRGB32F_IN).

Runs where the reference tree is present (oracle/_ref, the reference's
BVH/BVH2Common.cpp compiled in place).  Each case is a DX brick set of the
smooth union with 8 seeded words appended to every brick (RGB8 colours or
16-bit texture coordinates at the brick corners, the layouts' extra data,
BVH/BVH2Common.cpp:912-961), its BVH2, and the records the reference's
BVHRT::RayQuery_NearestHit returns for the rays of ref_rayquery.npz.

    python tests/golden/make_golden_layouts.py
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

OUT = os.path.join(HERE, "ref_layouts.npz")
LAYOUT_UV16, LAYOUT_RGB8 = 2 << 24, 3 << 24


def with_extra_words(hd, nodes, values, seed):
    """A DX set with 8 seeded words after every brick's packed distances."""
    rng = np.random.default_rng(seed)
    v_size = hd.brick_size + 2 * hd.brick_pad + 1
    vpi = 4 // hd.bytes_per_value
    words = (v_size ** 3 + vpi - 1) // vpi
    out_vals, out_nodes = [], nodes.copy()
    for i in range(nodes.shape[0]):
        out_nodes[i, 2] = i * (words + 8)
        out_vals.append(values[nodes[i, 2]:nodes[i, 2] + words])
        out_vals.append(rng.integers(0, 2 ** 32, 8, dtype=np.uint64).astype(np.uint32))
    return out_nodes, np.concatenate(out_vals).astype(np.uint32)


CASES = {
    "rgb8_q4": (LAYOUT_RGB8, 3, 4, 0, 4),
    "rgb8_q1pad": (LAYOUT_RGB8, 3, 4, 1, 1),
    "uv16_q2": (LAYOUT_UV16, 3, 4, 0, 2),
}


def build_case(name):
    layout, depth, bs, pad, bpv = CASES[name]
    hd, n, v = lrt.sbs_from_sdf(lrt.Sdf(**scenes.union_params()), depth, bs, pad, bpv)
    n2, v2 = with_extra_words(hd, n, v, seed=len(name))
    hdr = np.array([hd.brick_size, hd.brick_pad, hd.bytes_per_value, layout], np.uint32)
    return hdr, n2, v2


def main():
    gold = np.load(os.path.join(HERE, "ref_rayquery.npz"))
    P, D = gold["rays_pos"], gold["rays_dir"]
    out = {}
    for name in CASES:
        hdr, n, v = build_case(name)
        pairs, _, _ = lrt.build_bvh2(orc.node_boxes(n), 1)
        oh = orc.SbsHeader(*[int(x) for x in hdr])
        out[name + "_hdr"], out[name + "_nodes"], out[name + "_values"], out[name + "_pairs"] = hdr, n, v, pairs
        out[name + "_hits"] = ref.RefScene("sbs", (oh, n, v), pairs, (8, 2, 0, 0, 0, 1, 1)).query(P, D)
    # NORMAL_MODE_SDF_SMOOTHED on the neighbour layout (ID32F_IRGB32F_IN, create_grid_sbs)
    from litert_gb300 import dr
    hd, n, v, vf = dr.grid_sbs(6, 4, lrt.Sdf(**scenes.union_params()), None)
    pairs, _, _ = lrt.build_bvh2(orc.node_boxes(n), 1)
    oh = orc.SbsHeader(hd.brick_size, hd.brick_pad, hd.bytes_per_value, hd.aux_data)
    out["smooth_hdr"] = np.array([hd.brick_size, hd.brick_pad, hd.bytes_per_value, hd.aux_data], np.uint32)
    out["smooth_nodes"], out["smooth_values"], out["smooth_values_f"], out["smooth_pairs"] = n, v, vf, pairs
    for nm in (0, 2):
        out[f"smooth_hits_n{nm}"] = ref.RefScene("sbs", (oh, n, v, vf), pairs, (8, 2, nm, 0, 0, 1, 1)).query(P, D)
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, {k: v.shape for k, v in out.items() if k.endswith("_hits")})


if __name__ == "__main__":
    main()
