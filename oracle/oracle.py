"""ctypes binding of the CPU oracle (oracle/_build/liblrt_oracle.so).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and bench.py's
CPU baseline legs to verify the GPU engine against.  The product never imports
this module.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liblrt_oracle.so")

HIT_DTYPE = np.dtype([("t", "<f4"), ("primId", "<u4"), ("instId", "<u4"), ("geomId", "<u4"), ("coords", "<f4", (4,))])


class Preset(C.Structure):
    _fields_ = [("render_mode", C.c_uint32), ("sdf_node_intersect", C.c_uint32), ("normal_mode", C.c_uint32),
                ("ray_gen_mode", C.c_uint32), ("interpolation_mode", C.c_uint32),
                ("representation_mode", C.c_uint32), ("spp", C.c_uint32)]


class SbsHeader(C.Structure):
    _fields_ = [("brick_size", C.c_uint32), ("brick_pad", C.c_uint32), ("bytes_per_value", C.c_uint32),
                ("aux_data", C.c_uint32)]


VP = C.c_void_p


class OrcScene(C.Structure):
    _fields_ = [("type", C.c_uint32), ("sbs_hdr", SbsHeader), ("sbs_nodes", VP), ("n_sbs_nodes", C.c_uint32),
                ("sbs_values", VP), ("sbs_values_f", VP), ("svs_nodes", VP), ("n_svs_nodes", C.c_uint32),
                ("vert_pos4", VP), ("tri_indices", VP), ("prim_indices", VP), ("leaf_start_count", VP),
                ("pairs", VP), ("n_pairs", C.c_uint32), ("tri_indices_orig", VP),
                ("inst_bmin", C.c_float * 3), ("inst_bmax", C.c_float * 3),
                ("inst_inv", C.c_float * 16), ("inst_inv_t", C.c_float * 16), ("preset", Preset),
                ("closest_hit", C.c_int), ("seed", C.c_uint32)]


class Counters(C.Structure):
    _fields_ = [("n_fat", C.c_uint64), ("n_leaf", C.c_uint64), ("n_vox", C.c_uint64), ("n_vox_loaded", C.c_uint64),
                ("n_finder", C.c_uint64), ("n_tri", C.c_uint64)]


class SdfDesc(C.Structure):
    _fields_ = [("n_spheres", C.c_uint32), ("spheres", VP), ("n_boxes", C.c_uint32), ("boxes", VP), ("k", C.c_float)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"oracle library missing at {LIB_PATH}; run oracle/build.py")
        L = C.CDLL(LIB_PATH)
        L.orc_render.restype = Counters
        L.orc_render.argtypes = [C.POINTER(OrcScene), C.c_uint32, C.c_uint32, VP, VP, VP, VP, C.c_int]
        L.orc_render_pixels.restype = Counters
        L.orc_render_pixels.argtypes = [C.POINTER(OrcScene), C.c_uint32, C.c_uint32, VP, VP, VP, C.c_uint32, VP, C.c_int]
        L.orc_bvh2_build.restype = C.c_uint32
        L.orc_bvh2_build.argtypes = [VP, C.c_uint32, C.c_uint32, C.POINTER(VP), C.POINTER(VP), C.POINTER(VP),
                                     C.POINTER(C.c_uint32)]
        L.orc_free.argtypes = [VP]
        L.orc_build_sbs.restype = C.c_uint32
        L.orc_build_sbs.argtypes = [C.POINTER(SdfDesc), C.c_uint32, SbsHeader, C.POINTER(VP), C.POINTER(VP),
                                    C.POINTER(C.c_uint32)]
        L.orc_build_svs.restype = C.c_uint32
        L.orc_build_svs.argtypes = [C.POINTER(SdfDesc), C.c_uint32, C.POINTER(VP)]
        L.orc_sdf_eval.restype = C.c_float
        L.orc_sdf_eval.argtypes = [C.POINTER(SdfDesc), C.c_float, C.c_float, C.c_float]
        L.orc_ray_query_nearest.restype = None
        for n in ("orc_perspective",):
            getattr(L, n).argtypes = [C.c_float, C.c_float, C.c_float, C.c_float, VP]
        L.orc_look_at.argtypes = [VP, VP, VP, VP]
        L.orc_inverse4x4.argtypes = [VP, VP]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def _sdf_desc(spheres, boxes, k):
    spheres = np.ascontiguousarray(np.zeros((0, 4)) if spheres is None else spheres, np.float32).reshape(-1, 4)
    boxes = np.ascontiguousarray(np.zeros((0, 16)) if boxes is None else boxes, np.float32).reshape(-1, 16)
    d = SdfDesc(spheres.shape[0], _p(spheres), boxes.shape[0], _p(boxes), float(k))
    return d, (spheres, boxes)


def sdf_eval(spheres, boxes, k, p):
    d, keep = _sdf_desc(spheres, boxes, k)
    return lib().orc_sdf_eval(C.byref(d), float(p[0]), float(p[1]), float(p[2]))


def build_sbs(spheres, boxes, k, depth, brick_size, brick_pad=0, bytes_per_value=4):
    d, keep = _sdf_desc(spheres, boxes, k)
    hdr = SbsHeader(brick_size, brick_pad, bytes_per_value, 1 << 24)
    pn, pv, nv = VP(), VP(), C.c_uint32()
    n = lib().orc_build_sbs(C.byref(d), depth, hdr, C.byref(pn), C.byref(pv), C.byref(nv))
    nodes = np.ctypeslib.as_array(C.cast(pn, C.POINTER(C.c_uint32)), (max(n, 1) * 4,))[: n * 4].copy().reshape(-1, 4)
    values = np.ctypeslib.as_array(C.cast(pv, C.POINTER(C.c_uint32)), (max(nv.value, 1),))[: nv.value].copy()
    lib().orc_free(pn)
    lib().orc_free(pv)
    return hdr, nodes, values


def build_svs(spheres, boxes, k, depth):
    d, keep = _sdf_desc(spheres, boxes, k)
    pn = VP()
    n = lib().orc_build_svs(C.byref(d), depth, C.byref(pn))
    nodes = np.ctypeslib.as_array(C.cast(pn, C.POINTER(C.c_uint32)), (max(n, 1) * 4,))[: n * 4].copy().reshape(-1, 4)
    lib().orc_free(pn)
    return nodes


def eye_rays(w, h, proj_inv, wv_inv, pix, dx=0.5, dy=0.5):
    pix = np.ascontiguousarray(pix, np.uint32)
    pi = np.ascontiguousarray(proj_inv, np.float32).reshape(16)
    wi = np.ascontiguousarray(wv_inv, np.float32).reshape(16)
    pos = np.zeros((pix.size, 4), np.float32)
    dr = np.zeros((pix.size, 4), np.float32)
    lib().orc_eye_rays(C.c_uint32(w), C.c_uint32(h), _p(pi), _p(wi), _p(pix), C.c_uint32(pix.size), C.c_float(dx),
                       C.c_float(dy), _p(pos), _p(dr))
    return pos, dr


def node_boxes(nodes):
    """Per-node AABB exactly as AddGeom_SdfSBS / AddGeom_SdfSVS compute it
    (BVH/BVH2Common_host.cpp:546-555, 640-653), float32 arithmetic."""
    nodes = np.asarray(nodes, np.uint32).reshape(-1, 4)
    p = np.stack([(nodes[:, 0] >> 16), (nodes[:, 0] & 0xFFFF), (nodes[:, 1] >> 16)], 1).astype(np.float32)
    sz = (nodes[:, 1] & 0xFFFF).astype(np.float32)[:, None]
    lo = np.float32(-1) + (np.float32(2.0) * p) / sz
    hi = lo + (np.float32(2.0) * np.float32(1)) / sz
    return np.concatenate([lo, hi], 1).astype(np.float32)


def bvh2_build(boxes6, prims_in_leaf):
    boxes6 = np.ascontiguousarray(boxes6, np.float32).reshape(-1, 6)
    pp, psc, po, nl = VP(), VP(), VP(), C.c_uint32()
    n = lib().orc_bvh2_build(_p(boxes6), boxes6.shape[0], prims_in_leaf, C.byref(pp), C.byref(psc), C.byref(po), C.byref(nl))
    pairs = np.ctypeslib.as_array(C.cast(pp, C.POINTER(C.c_uint8)), (n * 64,)).copy()
    sc = np.ctypeslib.as_array(C.cast(psc, C.POINTER(C.c_uint32)), (max(nl.value, 1),))[: nl.value].copy()
    order = np.ctypeslib.as_array(C.cast(po, C.POINTER(C.c_uint32)), (boxes6.shape[0],)).copy()
    for q in (pp, psc, po):
        lib().orc_free(q)
    return pairs, sc, order


class Scene:
    """One geometry + identity-or-given instance, as the oracle sees it."""

    def __init__(self, kind, *, sbs=None, svs=None, mesh=None, pairs=None, matrix=None, closest_hit=True,
                 render_mode=1, intersect=2, representation_mode=1, spp=1, normal_mode=0, ray_gen_mode=0, seed=0):
        self.keep = []
        s = OrcScene()
        m = np.eye(4, dtype=np.float32) if matrix is None else np.asarray(matrix, np.float32)
        inv = np.linalg.inv(m.astype(np.float64)).astype(np.float32)
        s.inst_inv[:] = inv.reshape(16).tolist()
        s.inst_inv_t[:] = inv.T.reshape(16).tolist()
        if kind == "sbs":
            hdr, nodes, values = sbs[:3]
            values_f = sbs[3] if len(sbs) > 3 else None
            nodes = np.ascontiguousarray(nodes, np.uint32)
            values = np.ascontiguousarray(values, np.uint32)
            layout = hdr.aux_data & 0xFF000000
            # AddGeom_SdfSBS, BVH/BVH2Common_host.cpp:572-592
            s.type = 11 if layout in (3 << 24, 4 << 24, 5 << 24) else (10 if layout == 2 << 24 else 6)
            s.sbs_hdr = SbsHeader(hdr.brick_size, hdr.brick_pad, hdr.bytes_per_value, hdr.aux_data)
            s.sbs_nodes, s.n_sbs_nodes, s.sbs_values = _p(nodes), nodes.shape[0], _p(values)
            self.keep += [nodes, values]
            if values_f is not None:
                vf = np.ascontiguousarray(values_f, np.float32)
                s.sbs_values_f = _p(vf)
                self.keep.append(vf)
            boxes = node_boxes(nodes)
            gmin, gmax = np.array([-1, -1, -1], np.float32), np.array([1, 1, 1], np.float32)
            pil = 1
        elif kind == "svs":
            nodes = np.ascontiguousarray(svs, np.uint32)
            s.type = 5
            s.svs_nodes, s.n_svs_nodes = _p(nodes), nodes.shape[0]
            self.keep.append(nodes)
            boxes = node_boxes(nodes)
            gmin, gmax = np.array([-1, -1, -1], np.float32), np.array([1, 1, 1], np.float32)
            pil = 1
        else:
            vpos, idx = mesh
            vpos = np.asarray(vpos, np.float32)
            v4 = np.ones((vpos.shape[0], 4), np.float32)
            v4[:, :3] = vpos[:, :3]
            idx = np.ascontiguousarray(idx, np.uint32).reshape(-1, 3)
            tri = v4[idx][:, :, :3]
            boxes = np.concatenate([tri.min(1), tri.max(1)], 1).astype(np.float32)
            s.type = 0
            gmin, gmax = vpos[:, :3].min(0), vpos[:, :3].max(0)
            pil = 2
        if pairs is None:
            pairs_b, sc, order = bvh2_build(boxes, pil)
        else:
            pairs_b, sc, order = pairs
        pairs_b = np.ascontiguousarray(pairs_b)
        s.pairs, s.n_pairs = _p(pairs_b), pairs_b.nbytes // 64
        self.keep.append(pairs_b)
        if kind == "mesh":
            reord = np.ascontiguousarray(idx[order], np.uint32)
            order = np.ascontiguousarray(order, np.uint32)
            sc = np.ascontiguousarray(sc, np.uint32)
            idx_flat = np.ascontiguousarray(idx.reshape(-1))
            s.vert_pos4, s.tri_indices, s.prim_indices, s.leaf_start_count = _p(v4), _p(reord), _p(order), _p(sc)
            s.tri_indices_orig = _p(idx_flat)
            self.keep += [v4, reord, order, sc, idx_flat]
        # instance box: transformed corners of the geometry box
        corners = np.array([[gmax[0] if c & 1 else gmin[0], gmax[1] if c & 2 else gmin[1],
                             gmax[2] if c & 4 else gmin[2], 1.0] for c in range(8)], np.float32)
        tc = corners @ m.T
        s.inst_bmin[:] = tc[:, :3].min(0).tolist()
        s.inst_bmax[:] = tc[:, :3].max(0).tolist()
        s.preset = Preset(render_mode, intersect, normal_mode, ray_gen_mode, 0, representation_mode, spp)
        s.closest_hit = 1 if closest_hit else 0
        s.seed = seed & 0xFFFFFFFF
        self.s = s

    def render(self, w, h, proj_inv, wv_inv, hits=True, rgba=False, threads=0):
        pi = np.ascontiguousarray(proj_inv, np.float32).reshape(16)
        wi = np.ascontiguousarray(wv_inv, np.float32).reshape(16)
        hh = np.zeros(w * h, HIT_DTYPE) if hits else None
        col = np.zeros((w * h, 4), np.float32) if rgba else None
        cnt = lib().orc_render(C.byref(self.s), w, h, _p(pi), _p(wi), _p(hh), _p(col), threads)
        return hh, col, cnt

    def query_rays(self, pos_near, dir_far, threads=0):
        pos = np.ascontiguousarray(pos_near, np.float32).reshape(-1, 4)
        dr = np.ascontiguousarray(dir_far, np.float32).reshape(-1, 4)
        out = np.zeros(pos.shape[0], HIT_DTYPE)
        lib().orc_query_rays(C.byref(self.s), _p(pos), _p(dr), C.c_uint32(pos.shape[0]), _p(out), C.c_int(threads))
        return out

    def render_pixels(self, w, h, proj_inv, wv_inv, pix, threads=0):
        pi = np.ascontiguousarray(proj_inv, np.float32).reshape(16)
        wi = np.ascontiguousarray(wv_inv, np.float32).reshape(16)
        pix = np.ascontiguousarray(pix, np.uint32)
        hh = np.zeros(pix.size, HIT_DTYPE)
        cnt = lib().orc_render_pixels(C.byref(self.s), w, h, _p(pi), _p(wi), _p(pix), pix.size, _p(hh), threads)
        return hh, cnt
