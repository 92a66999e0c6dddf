"""Shared helpers for the parity tests: build a scene both ways and compare hits."""
import numpy as np

from litert_gb300 import lrt, scenes
from oracle import oracle as orc


def orc_header(h):
    return orc.SbsHeader(h.brick_size, h.brick_pad, h.bytes_per_value, h.aux_data)


def sbs_scene(sdf_params, depth, brick_size, pad=0, bpv=4):
    h, nodes, values = lrt.sbs_from_sdf(lrt.Sdf(**sdf_params), depth, brick_size, pad, bpv)
    return h, nodes, values


def gpu_scene_sbs(h, nodes, values, values_f=None, **preset):
    s = lrt.Scene(0)
    g = s.add_sbs(h, nodes, values, values_f)
    s.add_instance(g)
    s.commit_scene()
    if preset:
        s.set_preset(**preset)
    return s


def oracle_render(osc, view):
    w, h, wv, pj = view
    hits, col, cnt = osc.render(w, h, lrt.inverse4x4(pj), lrt.inverse4x4(wv), rgba=True)
    return hits, col, cnt


def compare_hits16(g, o):
    """g: HIT16 records from the GPU, o: full oracle hits.  Returns dict of mismatch counts."""
    miss_g = g["primId"] == lrt.MISS
    miss_o = o["primId"] == lrt.MISS
    both = ~miss_g & ~miss_o
    return dict(
        n=g.size,
        hits=int((~miss_o).sum()),
        mask=int((miss_g != miss_o).sum()),
        t=int((g["t"][both].view(np.uint32) != o["t"][both].view(np.uint32)).sum()),
        prim=int((g["primId"][both] != o["primId"][both]).sum()),
        nx=int((g["nx"][both].view(np.uint32) != o["coords"][both, 2].view(np.uint32)).sum()),
        ny=int((g["ny"][both].view(np.uint32) != o["coords"][both, 3].view(np.uint32)).sum()),
        max_dt=float(np.abs(g["t"][both] - o["t"][both]).max()) if both.any() else 0.0,
    )
