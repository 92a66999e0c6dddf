"""ctypes binding of oracle/_ref/libref_dr.so: the reference's own
MultiRendererDR (RenderDR with the border integral, OptimizeStepAdam,
OptimizeFixedStructure), create_grid_sbs and the SDF -> SBS / SVS builders
(utils/sparse_octree_builder.cpp), compiled in place (see oracle/build_ref.py
and oracle/ref_driver_dr.cpp).  Test infrastructure: used to pin the oracle's
restatements and to generate tests/golden/ fixtures.  Available only where the
reference tree is.
"""
import ctypes as C
import os

import numpy as np

from . import build_ref
from . import oracle as orc
from .oracle import SbsHeader

VP = C.c_void_p
SDF_FN = C.CFUNCTYPE(C.c_float, VP, C.c_float, C.c_float, C.c_float)
_lib = None


class DrSettings(C.Structure):
    """RefDrSettings of oracle/ref_driver_dr.cpp: the MultiRendererDRPreset fields a test varies."""
    _fields_ = [(k, C.c_uint32) for k in ("render_mode", "reconstruction_flags", "loss_function", "input_type",
                                          "border_sampling", "raycasting_mask", "spp", "border_spp", "iterations",
                                          "image_batch_size", "reg_function", "redistancing_enable")] + \
               [(k, C.c_float) for k in ("border_relax_eps", "lr", "reg_lambda", "reg_power")]


def available():
    return build_ref.available() or os.path.exists(build_ref.DR_LIB)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(build_ref.DR_LIB):
            if build_ref.build_dr() is None:
                raise RuntimeError("reference tree not present; the in-place reference build is unavailable")
        L = C.CDLL(build_ref.DR_LIB)
        L.ref_build_sbs.restype = VP
        L.ref_build_sbs.argtypes = [VP, VP, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32]
        L.ref_build_svs.restype = VP
        L.ref_build_svs.argtypes = [VP, VP, C.c_uint32, C.c_uint32, C.POINTER(C.c_uint32)]
        L.ref_svs_copy.argtypes = [VP, VP]
        L.ref_svs_free.argtypes = [VP]
        L.ref_grid_sbs.restype = VP
        L.ref_grid_sbs.argtypes = [C.c_uint32, C.c_uint32, C.c_float, C.c_float, C.c_float, C.c_float, C.c_uint32]
        L.ref_sbs_sizes.argtypes = [VP, C.POINTER(SbsHeader), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                    C.POINTER(C.c_uint32)]
        L.ref_sbs_copy.argtypes = [VP, VP, VP, VP]
        L.ref_sbs_free.argtypes = [VP]
        L.ref_dr_optimize.argtypes = [C.POINTER(SbsHeader), VP, C.c_uint32, VP, C.c_uint32, VP, C.c_uint32, VP,
                                      C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, VP, VP, VP,
                                      C.POINTER(DrSettings), C.c_uint32, VP, VP, VP]
        L.ref_render_float.argtypes = [C.POINTER(SbsHeader), VP, C.c_uint32, VP, C.c_uint32, VP, C.c_uint32,
                                       C.c_uint32, C.c_uint32, VP, VP, C.c_uint32, C.c_uint32, C.c_uint32,
                                       C.c_uint32, C.c_uint32, VP]
        L.ref_dr_adam.argtypes = [C.c_uint32, VP, VP, VP, C.c_uint32, C.c_float, C.c_float, C.c_float, C.c_float]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def _take_sbs(h):
    L = lib()
    hdr, nn, nv, nf = SbsHeader(), C.c_uint32(), C.c_uint32(), C.c_uint32()
    L.ref_sbs_sizes(h, C.byref(hdr), C.byref(nn), C.byref(nv), C.byref(nf))
    nodes = np.zeros((nn.value, 4), np.uint32)
    values = np.zeros(nv.value, np.uint32)
    values_f = np.zeros(max(nf.value, 1), np.float32)
    L.ref_sbs_copy(h, _p(nodes), _p(values), _p(values_f))
    L.ref_sbs_free(h)
    return hdr, nodes, values, values_f[: nf.value]


def _sdf_callback(spheres, boxes, k):
    """The oracle's analytic SDF (orc_sdf_eval) handed to the reference builder."""
    desc, keep = orc._sdf_desc(spheres, boxes, k)
    fn = C.cast(orc.lib().orc_sdf_eval, VP)
    return fn, desc, keep


def build_sbs(spheres, boxes, k, depth, brick_size, brick_pad=0, bytes_per_value=4, threads=1):
    """create_sdf_SBS of the reference on the oracle's SDF: (header, nodes, values)."""
    fn, desc, keep = _sdf_callback(spheres, boxes, k)
    h = lib().ref_build_sbs(fn, C.cast(C.pointer(desc), VP), depth, brick_size, brick_pad, bytes_per_value, threads)
    hdr, nodes, values, _ = _take_sbs(h)
    return hdr, nodes, values


def build_svs(spheres, boxes, k, depth, threads=1):
    fn, desc, keep = _sdf_callback(spheres, boxes, k)
    n = C.c_uint32()
    h = lib().ref_build_svs(fn, C.cast(C.pointer(desc), VP), depth, threads, C.byref(n))
    nodes = np.zeros((n.value, 4), np.uint32)
    lib().ref_svs_copy(h, _p(nodes))
    lib().ref_svs_free(h)
    return nodes


def grid_sbs(brick_count, brick_size, center, radius, gradient_colors):
    """create_grid_sbs(circle_sdf(center, radius), single_color or gradient_color)."""
    h = lib().ref_grid_sbs(brick_count, brick_size, float(center[0]), float(center[1]), float(center[2]),
                           float(radius), 1 if gradient_colors else 0)
    return _take_sbs(h)


def settings(render_mode=1, reconstruction_flags=3, loss_function=0, input_type=0, border_sampling=0,
             raycasting_mask=0, spp=1, border_spp=256, iterations=1, image_batch_size=1, reg_function=0,
             redistancing_enable=0, border_relax_eps=1e-3, lr=3e-3, reg_lambda=0.25, reg_power=2.0):
    s = DrSettings()
    for k, v in dict(locals()).items():
        if k != "s":
            setattr(s, k, v)
    return s


def optimize(hdr, nodes, values, params, pairs, images, world_views, projs, st, seed):
    """MultiRendererDR::OptimizeFixedStructure on the reference (one thread):
    returns (params after, last gradient, last images)."""
    nodes = np.ascontiguousarray(nodes, np.uint32)
    values = np.ascontiguousarray(values, np.uint32)
    params = np.ascontiguousarray(params, np.float32)
    pairs = np.ascontiguousarray(pairs)
    imgs = np.ascontiguousarray(np.stack([np.asarray(i, np.float32).reshape(-1, 4) for i in images]))
    nv, h_, w_ = len(images), images[0].shape[0], images[0].shape[1]
    wv = np.ascontiguousarray(np.stack([np.asarray(m, np.float32).reshape(16) for m in world_views]))
    pj = np.ascontiguousarray(np.stack([np.asarray(m, np.float32).reshape(16) for m in projs]))
    out_p = np.zeros_like(params)
    out_g = np.zeros_like(params)
    out_i = np.zeros_like(imgs)
    h = SbsHeader(hdr.brick_size, hdr.brick_pad, hdr.bytes_per_value, hdr.aux_data)
    lib().ref_dr_optimize(C.byref(h), _p(nodes), nodes.shape[0], _p(values), values.size, _p(params), params.size,
                          _p(pairs), pairs.nbytes // 64, nv, w_, h_, _p(imgs), _p(wv), _p(pj), C.byref(st), seed,
                          _p(out_p), _p(out_g), _p(out_i))
    return out_p, out_g, out_i.reshape(nv, h_, w_, 4)


def adam(it, g, x, state, lr, b1=0.9, b2=0.999, eps=1e-8):
    """OptimizeStepAdam of the reference on x and state (updated in place)."""
    g = np.ascontiguousarray(g, np.float32)
    lib().ref_dr_adam(it, _p(g), _p(x), _p(state), x.size, lr, b1, b2, eps)


def render_float(hdr, nodes, values, pairs, view, render_mode, intersect, spp, ray_gen_mode, seed):
    """MultiRenderer::RenderFloat of the reference (one thread): (H, W, 4) colours."""
    w, h, wv, pj = view
    nodes = np.ascontiguousarray(nodes, np.uint32)
    values = np.ascontiguousarray(values, np.uint32)
    pairs = np.ascontiguousarray(pairs)
    out = np.zeros((h, w, 4), np.float32)
    wv = np.ascontiguousarray(wv, np.float32).reshape(16)
    pj = np.ascontiguousarray(pj, np.float32).reshape(16)
    hh = SbsHeader(hdr.brick_size, hdr.brick_pad, hdr.bytes_per_value, hdr.aux_data)
    lib().ref_render_float(C.byref(hh), _p(nodes), nodes.shape[0], _p(values), values.size, _p(pairs),
                           pairs.nbytes // 64, w, h, _p(wv), _p(pj), render_mode, intersect, spp, ray_gen_mode,
                           seed, _p(out))
    return out
