"""Shared helpers for the parity tests: build a scene both ways and compare hits."""
import numpy as np

from litert_gb300 import lrt, scenes
from oracle import oracle as orc


def orc_header(h):
    return orc.SbsHeader(h.brick_size, h.brick_pad, h.bytes_per_value, h.aux_data)


def sbs_scene(sdf_params, depth, brick_size, pad=0, bpv=4):
    h, nodes, values = lrt.sbs_from_sdf(lrt.Sdf(**sdf_params), depth, brick_size, pad, bpv)
    return h, nodes, values


def gpu_scene_sbs(h, nodes, values, values_f=None, variant=None, **preset):
    s = lrt.Scene(0)
    if variant is not None:
        s.set_tuning("variant", variant)
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


def canon_bits(a):
    """Float32 bit patterns with every NaN mapped to one pattern (CPU and GPU
    produce different NaN payloads, e.g. the normal of a zero gradient)."""
    a = np.ascontiguousarray(a, np.float32)
    b = a.view(np.uint32).copy()
    b[np.isnan(a)] = 0x7FC00000
    return b


def records_equal(ga, oa):
    """Bitwise equality of structured hit arrays, NaN == NaN."""
    fa = np.ascontiguousarray(ga).view(np.float32)
    fb = np.ascontiguousarray(oa).view(np.float32)
    return np.array_equal(canon_bits(fa), canon_bits(fb))


def compare_hits16(g, o):
    """g: HIT16 records from the GPU, o: full oracle hits.  Returns dict of mismatch counts."""
    miss_g = g["primId"] == lrt.MISS
    miss_o = o["primId"] == lrt.MISS
    both = ~miss_g & ~miss_o
    return dict(
        n=g.size,
        hits=int((~miss_o).sum()),
        mask=int((miss_g != miss_o).sum()),
        t=int((canon_bits(g["t"][both]) != canon_bits(o["t"][both])).sum()),
        prim=int((g["primId"][both] != o["primId"][both]).sum()),
        nx=int((canon_bits(g["nx"][both]) != canon_bits(o["coords"][both, 2])).sum()),
        ny=int((canon_bits(g["ny"][both]) != canon_bits(o["coords"][both, 3])).sum()),
        max_dt=float(np.abs(g["t"][both] - o["t"][both]).max()) if both.any() else 0.0,
    )
