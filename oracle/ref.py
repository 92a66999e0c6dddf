"""ctypes binding of oracle/_ref/libref_bvh.so: the reference's own
BVHRT::RayQuery_NearestHit, dr::BVHDR::RayQuery_NearestHitWithGrad and
eye-ray code compiled in place (see
oracle/build_ref.py).  Test infrastructure: used to pin the oracle and to
generate tests/golden/ fixtures.  Available only where the reference tree is.
"""
import ctypes as C
import os

import numpy as np

from . import build_ref
from .oracle import HIT_DTYPE, Preset, SbsHeader

VP = C.c_void_p
_lib = None


def available():
    return build_ref.available() or os.path.exists(build_ref.LIB)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(build_ref.LIB):
            if build_ref.build() is None:
                raise RuntimeError("reference tree not present; the in-place reference build is unavailable")
        L = C.CDLL(build_ref.LIB)
        L.ref_make_sbs.restype = VP
        L.ref_make_sbs.argtypes = [C.POINTER(SbsHeader), VP, C.c_uint32, VP, C.c_uint32, VP, C.c_uint32, VP,
                                   C.c_uint32, C.POINTER(Preset)]
        L.ref_make_svs.restype = VP
        L.ref_make_svs.argtypes = [VP, C.c_uint32, VP, C.c_uint32, C.POINTER(Preset)]
        L.ref_make_tris.restype = VP
        L.ref_make_tris.argtypes = [VP, C.c_uint32, VP, C.c_uint32, VP, VP, C.c_uint32, VP, C.c_uint32,
                                    C.POINTER(Preset)]
        L.ref_free.argtypes = [VP]
        L.ref_query.argtypes = [VP, VP, VP, C.c_uint32, VP]
        L.ref_eye_rays.argtypes = [C.c_uint32, C.c_uint32, VP, VP, VP, C.c_uint32, C.c_float, C.c_float, VP, VP]
        L.ref_dr_query.argtypes = [VP, C.c_uint32, VP, VP, C.c_uint32, VP]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


class RefScene:
    """A BVHRT of the reference holding one geometry and an identity instance."""

    def __init__(self, kind, data, pairs, preset):
        self.keep = [pairs]
        pairs = np.ascontiguousarray(pairs)
        npairs = pairs.nbytes // 64
        pr = Preset(*preset)
        self.keep.append(pr)
        if kind == "sbs":
            hdr, nodes, values = data[:3]
            vf = data[3] if len(data) > 3 else None
            nodes = np.ascontiguousarray(nodes, np.uint32)
            values = np.ascontiguousarray(values, np.uint32)
            h = SbsHeader(hdr.brick_size, hdr.brick_pad, hdr.bytes_per_value, hdr.aux_data)
            vfa = None if vf is None else np.ascontiguousarray(vf, np.float32)
            self.keep += [nodes, values, h, vfa]
            self.h = lib().ref_make_sbs(C.byref(h), _p(nodes), nodes.shape[0], _p(values), values.size, _p(vfa),
                                        0 if vfa is None else vfa.size, _p(pairs), npairs, C.byref(pr))
        elif kind == "svs":
            nodes = np.ascontiguousarray(data, np.uint32)
            self.keep.append(nodes)
            self.h = lib().ref_make_svs(_p(nodes), nodes.shape[0], _p(pairs), npairs, C.byref(pr))
        else:
            vpos4, idx, order, sc = data
            vpos4 = np.ascontiguousarray(vpos4, np.float32)
            idx = np.ascontiguousarray(idx, np.uint32)
            order = np.ascontiguousarray(order, np.uint32)
            sc = np.ascontiguousarray(sc, np.uint32)
            self.keep += [vpos4, idx, order, sc]
            self.h = lib().ref_make_tris(_p(vpos4), vpos4.shape[0], _p(idx), idx.size // 3, _p(order), _p(sc),
                                         sc.size, _p(pairs), npairs, C.byref(pr))

    def query(self, pos_near, dir_far):
        pos = np.ascontiguousarray(pos_near, np.float32).reshape(-1, 4)
        dr = np.ascontiguousarray(dir_far, np.float32).reshape(-1, 4)
        out = np.zeros(pos.shape[0], HIT_DTYPE)
        lib().ref_query(self.h, _p(pos), _p(dr), pos.shape[0], _p(out))
        return out

    def dr_query(self, flags, pos_near, dir_far):
        """dr::BVHDR::RayQuery_NearestHitWithGrad records (oracle.oracle_dr.RECORD_DTYPE)."""
        from .oracle_dr import RECORD_DTYPE
        pos = np.ascontiguousarray(pos_near, np.float32).reshape(-1, 4)
        dr = np.ascontiguousarray(dir_far, np.float32).reshape(-1, 4)
        out = np.zeros(pos.shape[0], RECORD_DTYPE)
        lib().ref_dr_query(self.h, flags, _p(pos), _p(dr), pos.shape[0], _p(out))
        return out

    def __del__(self):
        if getattr(self, "h", None):
            lib().ref_free(self.h)
            self.h = None


def eye_rays(w, h, proj_inv, wv_inv, pix, dx=0.5, dy=0.5):
    pix = np.ascontiguousarray(pix, np.uint32)
    pi = np.ascontiguousarray(proj_inv, np.float32).reshape(16)
    wi = np.ascontiguousarray(wv_inv, np.float32).reshape(16)
    pos = np.zeros((pix.size, 4), np.float32)
    dr = np.zeros((pix.size, 4), np.float32)
    lib().ref_eye_rays(w, h, _p(pi), _p(wi), _p(pix), pix.size, dx, dy, _p(pos), _p(dr))
    return pos, dr
