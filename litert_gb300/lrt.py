"""Python host mirror of the lrt C ABI (include/lrt_gpu.h).

The classes follow the reference's interfaces for the hot path:
``Scene`` mirrors ISceneObject/BVHRT (ClearGeom, AddGeom_SdfSBS, AddGeom_SdfSVS,
AddGeom_Triangles3f, ClearScene, AddInstance, CommitScene, RayQuery_NearestHit,
BVH/BVH2Common.h:100-173) and ``Scene.render`` mirrors MultiRenderer::Render /
RenderFloat (Renderer/eye_ray_host.cpp:563-585) batched over views.  Errors from
the library raise ``LrtError``; there is no CPU fallback: if the compiled
engine is missing, loading fails.
"""
import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "liblrt_gb300.so")

# ---------------------------------------------------------------- enums (render_settings.h)
TYPE_MESH_TRIANGLE, TYPE_SDF_SVS, TYPE_SDF_SBS, TYPE_SDF_SBS_COL = 0, 5, 6, 11
RENDER_MODE_MASK, RENDER_MODE_LAMBERT_NO_TEX, RENDER_MODE_DEPTH, RENDER_MODE_LINEAR_DEPTH = 0, 1, 2, 3
RENDER_MODE_INVERSE_LINEAR_DEPTH, RENDER_MODE_NORMAL, RENDER_MODE_LAMBERT = 4, 8, 17
RENDER_MODE_PRIMITIVE, RENDER_MODE_TYPE, RENDER_MODE_GEOM, RENDER_MODE_BARYCENTRIC = 5, 6, 7, 9
RENDER_MODE_ST_ITERATIONS, RENDER_MODE_PHONG_NO_TEX, RENDER_MODE_DIFFUSE = 10, 12, 16
RENDER_MODE_PHONG, RENDER_MODE_HSV_DEPTH = 18, 19
INTERSECT_ST, INTERSECT_ANALYTIC, INTERSECT_NEWTON, INTERSECT_BBOX, INTERSECT_IT = 0, 1, 2, 3, 4
SBS_LAYOUT_DX = 1 << 24
SBS_LAYOUT_ID32F_IRGB32F = 4 << 24
SBS_LAYOUT_ID32F_IRGB32F_IN = 5 << 24
MISS = 0xFFFFFFFF

STATUS = {0: "ok", 1: "invalid argument", 2: "out of memory", 3: "CUDA error", 4: "unsupported",
          5: "device wait timed out", 6: "device bounds check failed", 7: "bad call order"}


class LrtError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"lrt error {status} ({STATUS.get(status, '?')}): {msg}")
        self.status = status


# ---------------------------------------------------------------- POD types (include/lrt_types.h)
class SbsHeader(C.Structure):
    _fields_ = [("brick_size", C.c_uint32), ("brick_pad", C.c_uint32), ("bytes_per_value", C.c_uint32),
                ("aux_data", C.c_uint32)]


class Preset(C.Structure):
    _fields_ = [("render_mode", C.c_uint32), ("sdf_node_intersect", C.c_uint32), ("normal_mode", C.c_uint32),
                ("ray_gen_mode", C.c_uint32), ("interpolation_mode", C.c_uint32),
                ("representation_mode", C.c_uint32), ("spp", C.c_uint32)]


class View(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("world_view", C.c_float * 16),
                ("proj", C.c_float * 16)]


class TuningChoice(C.Structure):
    _fields_ = [("variant", C.c_int), ("block_warps", C.c_int), ("stage", C.c_int), ("tile_w", C.c_int),
                ("stack", C.c_int), ("ms", C.c_float)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class SdfDesc(C.Structure):
    _fields_ = [("n_spheres", C.c_uint32), ("spheres", C.POINTER(C.c_float)), ("n_boxes", C.c_uint32),
                ("boxes", C.POINTER(C.c_float)), ("k", C.c_float)]


HIT_DTYPE = np.dtype([("t", "<f4"), ("primId", "<u4"), ("instId", "<u4"), ("geomId", "<u4"), ("coords", "<f4", (4,))])
HIT16_DTYPE = np.dtype([("t", "<f4"), ("primId", "<u4"), ("nx", "<f4"), ("ny", "<f4")])
BVH_PAIR_DTYPE = np.dtype([("lmin", "<f4", (3,)), ("lleft", "<u4"), ("lmax", "<f4", (3,)), ("lesc", "<u4"),
                           ("rmin", "<f4", (3,)), ("rleft", "<u4"), ("rmax", "<f4", (3,)), ("resc", "<u4")])

_lib = None


def lib():
    """Load the compiled engine.  Raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"lrt engine library missing at {LIB_PATH}; run litert_gb300.build.build()")
        L = C.CDLL(LIB_PATH)
        P, U32, I, VP = C.c_void_p, C.c_uint32, C.c_int, C.c_void_p
        sig = {
            "lrt_create": (I, [C.POINTER(P), I]),
            "lrt_destroy": (None, [P]),
            "lrt_last_error": (C.c_char_p, [P]),
            "lrt_status_string": (C.c_char_p, [I]),
            "lrt_clear_geom": (I, [P]),
            "lrt_add_sbs": (I, [P, C.POINTER(SbsHeader), VP, U32, VP, U32, VP, U32, C.POINTER(U32)]),
            "lrt_add_svs": (I, [P, VP, U32, C.POINTER(U32)]),
            "lrt_add_triangles": (I, [P, VP, C.c_size_t, C.c_size_t, VP, C.c_size_t, C.POINTER(U32)]),
            "lrt_clear_scene": (I, [P]),
            "lrt_add_instance": (I, [P, U32, VP, C.POINTER(U32)]),
            "lrt_commit_scene": (I, [P]),
            "lrt_set_preset": (I, [P, C.POINTER(Preset)]),
            "lrt_query_rays": (I, [P, VP, VP, U32, VP, I, VP]),
            "lrt_render": (I, [P, VP, U32, VP, VP, VP, VP]),
            "lrt_render_host": (I, [P, VP, U32, VP, VP, VP]),
            "lrt_last_launch_count": (U32, [P]),
            "lrt_render_counters": (I, [P, VP, U32, VP]),
            "lrt_get_bvh2": (I, [P, C.POINTER(VP), C.POINTER(U32)]),
            "lrt_sbs_build_from_sdf": (I, [C.POINTER(SdfDesc), U32, C.POINTER(SbsHeader), I, C.POINTER(P)]),
            "lrt_sbs_data": (I, [P, C.POINTER(SbsHeader), C.POINTER(VP), C.POINTER(U32), C.POINTER(VP), C.POINTER(U32)]),
            "lrt_sbs_free": (None, [P]),
            "lrt_svs_build_from_sdf": (I, [C.POINTER(SdfDesc), U32, I, C.POINTER(P)]),
            "lrt_sbs_build_from_sdf_gpu": (I, [I, C.POINTER(SdfDesc), U32, C.POINTER(SbsHeader), C.POINTER(P)]),
            "lrt_svs_build_from_sdf_gpu": (I, [I, C.POINTER(SdfDesc), U32, C.POINTER(P)]),
            "lrt_build_last_error": (C.c_char_p, []),
            "lrt_sbs_save": (I, [C.c_char_p, C.POINTER(SbsHeader), VP, U32, VP, U32]),
            "lrt_sbs_load": (I, [C.c_char_p, C.POINTER(P)]),
            "lrt_svs_save": (I, [C.c_char_p, VP, U32]),
            "lrt_svs_load": (I, [C.c_char_p, C.POINTER(P)]),
            "lrt_svs_data": (I, [P, C.POINTER(VP), C.POINTER(U32)]),
            "lrt_svs_free": (None, [P]),
            "lrt_perspective": (None, [C.c_float, C.c_float, C.c_float, C.c_float, VP]),
            "lrt_look_at": (None, [VP, VP, VP, VP]),
            "lrt_inverse4x4": (None, [VP, VP]),
            "lrt_build_bvh2": (I, [VP, U32, U32, C.POINTER(VP), C.POINTER(U32), C.POINTER(VP), C.POINTER(U32),
                                   C.POINTER(VP)]),
            "lrt_free": (None, [VP]),
            "lrt_set_tuning": (I, [P, C.c_char_p, I]),
            "lrt_refit_triangles": (I, [P, VP, C.c_size_t, C.c_size_t]),
            "lrt_render_noalloc": (I, [P, VP, U32, VP, VP, VP, VP]),
            "lrt_autotune": (I, [P, VP, U32, U32, C.POINTER(TuningChoice), VP, U32, C.POINTER(U32)]),
            "lrt_render_graph_create": (I, [P, VP, U32, VP, VP, VP, C.POINTER(P)]),
            "lrt_render_graph_launch": (I, [P, P, VP]),
            "lrt_render_graph_set_views": (I, [P, P, VP, U32]),
            "lrt_render_graph_destroy": (None, [P]),
            "lrt_set_seed": (I, [P, U32]),
            "lrt_set_bvh2": (I, [P, VP, U32]),
            "lrt_update_instance": (I, [P, U32, VP]),
            "lrt_update_geom_triangles": (I, [P, U32, VP, C.c_size_t, VP, C.c_size_t, C.c_size_t]),
            "lrt_add_aabb": (I, [P, U32, VP, C.c_size_t, C.POINTER(U32)]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


# ---------------------------------------------------------------- camera helpers
def perspective(fov_deg, aspect, znear, zfar):
    out = np.zeros(16, np.float32)
    lib().lrt_perspective(fov_deg, aspect, znear, zfar, _ptr(out))
    return out.reshape(4, 4)


def look_at(eye, center, up):
    out = np.zeros(16, np.float32)
    e, c, u = (np.ascontiguousarray(v, np.float32) for v in (eye, center, up))
    lib().lrt_look_at(_ptr(e), _ptr(c), _ptr(u), _ptr(out))
    return out.reshape(4, 4)


def inverse4x4(m):
    m = np.ascontiguousarray(m, np.float32).reshape(16)
    out = np.zeros(16, np.float32)
    lib().lrt_inverse4x4(_ptr(m), _ptr(out))
    return out.reshape(4, 4)


def make_views(views):
    """views: list of (width, height, world_view 4x4, proj 4x4) -> ctypes array."""
    arr = (View * len(views))()
    for i, (w, h, wv, pj) in enumerate(views):
        arr[i].width = int(w)
        arr[i].height = int(h)
        arr[i].world_view[:] = [float(x) for x in np.asarray(wv, np.float32).reshape(16)]
        arr[i].proj[:] = [float(x) for x in np.asarray(pj, np.float32).reshape(16)]
    return arr


# ---------------------------------------------------------------- scene construction
class Sdf:
    """Smooth union of spheres (n,4) and rounded boxes (m,16); see lrt_sdf_desc."""

    def __init__(self, spheres=None, boxes=None, k=0.0):
        self.spheres = np.ascontiguousarray(np.zeros((0, 4)) if spheres is None else spheres, np.float32).reshape(-1, 4)
        self.boxes = np.ascontiguousarray(np.zeros((0, 16)) if boxes is None else boxes, np.float32).reshape(-1, 16)
        self.k = float(k)

    def desc(self):
        d = SdfDesc()
        d.n_spheres = self.spheres.shape[0]
        d.spheres = self.spheres.ctypes.data_as(C.POINTER(C.c_float))
        d.n_boxes = self.boxes.shape[0]
        d.boxes = self.boxes.ctypes.data_as(C.POINTER(C.c_float))
        d.k = self.k
        return d


def _check(status, ctx=None, what=""):
    if status != 0:
        msg = lib().lrt_last_error(ctx).decode() if ctx else what
        raise LrtError(status, msg or what)


def _build_check(status, what):
    if status != 0:
        msg = lib().lrt_build_last_error()
        raise LrtError(status, (msg.decode() if msg else "") or what)


def sbs_from_sdf(sdf, depth, brick_size, brick_pad=0, bytes_per_value=4, threads=0, gpu=None):
    """create_sdf_SBS (utils/sdf_converter.cpp:162-181): returns (header, nodes (n,4) u32, values u32).
    gpu=<device index> builds on that GPU (depth >= 4; identical output)."""
    hdr = SbsHeader(brick_size, brick_pad, bytes_per_value, SBS_LAYOUT_DX)
    h = C.c_void_p()
    if gpu is not None:
        _build_check(lib().lrt_sbs_build_from_sdf_gpu(int(gpu), C.byref(sdf.desc()), depth, C.byref(hdr), C.byref(h)),
                     "lrt_sbs_build_from_sdf_gpu")
    else:
        _check(lib().lrt_sbs_build_from_sdf(C.byref(sdf.desc()), depth, C.byref(hdr), threads, C.byref(h)),
               what="lrt_sbs_build_from_sdf")
    try:
        oh, np_, nn, vp, nv = SbsHeader(), C.c_void_p(), C.c_uint32(), C.c_void_p(), C.c_uint32()
        _check(lib().lrt_sbs_data(h, C.byref(oh), C.byref(np_), C.byref(nn), C.byref(vp), C.byref(nv)))
        nodes = np.ctypeslib.as_array(C.cast(np_, C.POINTER(C.c_uint32)), (nn.value * 4,)).copy().reshape(-1, 4)
        values = np.ctypeslib.as_array(C.cast(vp, C.POINTER(C.c_uint32)), (nv.value,)).copy()
    finally:
        lib().lrt_sbs_free(h)
    return oh, nodes, values


def svs_from_sdf(sdf, depth, threads=0, gpu=None):
    """create_sdf_SVS (utils/sdf_converter.cpp:118-134): returns nodes (n,4) u32.
    gpu=<device index> builds on that GPU (depth >= 4; identical output)."""
    h = C.c_void_p()
    if gpu is not None:
        _build_check(lib().lrt_svs_build_from_sdf_gpu(int(gpu), C.byref(sdf.desc()), depth, C.byref(h)),
                     "lrt_svs_build_from_sdf_gpu")
    else:
        _check(lib().lrt_svs_build_from_sdf(C.byref(sdf.desc()), depth, threads, C.byref(h)),
               what="lrt_svs_build_from_sdf")
    try:
        np_, nn = C.c_void_p(), C.c_uint32()
        _check(lib().lrt_svs_data(h, C.byref(np_), C.byref(nn)))
        nodes = np.ctypeslib.as_array(C.cast(np_, C.POINTER(C.c_uint32)), (nn.value * 4,)).copy().reshape(-1, 4)
    finally:
        lib().lrt_svs_free(h)
    return nodes


def _sbs_arrays(h):
    oh, np_, nn, vp, nv = SbsHeader(), C.c_void_p(), C.c_uint32(), C.c_void_p(), C.c_uint32()
    _check(lib().lrt_sbs_data(h, C.byref(oh), C.byref(np_), C.byref(nn), C.byref(vp), C.byref(nv)))
    nodes = (np.ctypeslib.as_array(C.cast(np_, C.POINTER(C.c_uint32)), (nn.value * 4,)).copy() if nn.value
             else np.zeros(0, np.uint32))
    values = (np.ctypeslib.as_array(C.cast(vp, C.POINTER(C.c_uint32)), (nv.value,)).copy() if nv.value
              else np.zeros(0, np.uint32))
    return oh, nodes.reshape(-1, 4), values


def save_sbs(path, hdr, nodes, values):
    """save_sdf_SBS (sdfScene/sdf_scene.cpp:148-158)."""
    nodes = np.ascontiguousarray(nodes, np.uint32).reshape(-1, 4)
    values = np.ascontiguousarray(values, np.uint32)
    _check(lib().lrt_sbs_save(os.fsencode(path), C.byref(hdr), _ptr(nodes), nodes.shape[0], _ptr(values), values.size),
           what="lrt_sbs_save")


def load_sbs(path):
    """load_sdf_SBS (sdfScene/sdf_scene.cpp:160-173): (header, nodes (n,4) u32, values u32)."""
    h = C.c_void_p()
    _check(lib().lrt_sbs_load(os.fsencode(path), C.byref(h)), what="lrt_sbs_load")
    try:
        return _sbs_arrays(h)
    finally:
        lib().lrt_sbs_free(h)


def save_svs(path, nodes):
    """save_sdf_SVS (sdfScene/sdf_scene.cpp:121-127)."""
    nodes = np.ascontiguousarray(nodes, np.uint32).reshape(-1, 4)
    _check(lib().lrt_svs_save(os.fsencode(path), _ptr(nodes), nodes.shape[0]), what="lrt_svs_save")


def load_svs(path):
    """load_sdf_SVS (sdfScene/sdf_scene.cpp:129-137): nodes (n,4) u32."""
    h = C.c_void_p()
    _check(lib().lrt_svs_load(os.fsencode(path), C.byref(h)), what="lrt_svs_load")
    try:
        np_, nn = C.c_void_p(), C.c_uint32()
        _check(lib().lrt_svs_data(h, C.byref(np_), C.byref(nn)))
        if nn.value == 0:
            return np.zeros((0, 4), np.uint32)
        return np.ctypeslib.as_array(C.cast(np_, C.POINTER(C.c_uint32)), (nn.value * 4,)).copy().reshape(-1, 4)
    finally:
        lib().lrt_svs_free(h)


def build_bvh2(boxes6, prims_per_leaf):
    """The product's BVH builder on the host: (pairs bytes (n*64,), leaf_start_count, order)."""
    boxes6 = np.ascontiguousarray(boxes6, np.float32).reshape(-1, 6)
    pp, npairs, psc, nl, po = C.c_void_p(), C.c_uint32(), C.c_void_p(), C.c_uint32(), C.c_void_p()
    _check(lib().lrt_build_bvh2(_ptr(boxes6), boxes6.shape[0], prims_per_leaf, C.byref(pp), C.byref(npairs),
                                C.byref(psc), C.byref(nl), C.byref(po)), what="lrt_build_bvh2")
    pairs = np.ctypeslib.as_array(C.cast(pp, C.POINTER(C.c_uint8)), (npairs.value * 64,)).copy()
    sc = np.ctypeslib.as_array(C.cast(psc, C.POINTER(C.c_uint32)), (max(nl.value, 1),))[: nl.value].copy()
    order = np.ctypeslib.as_array(C.cast(po, C.POINTER(C.c_uint32)), (boxes6.shape[0],)).copy()
    for q in (pp, psc, po):
        lib().lrt_free(q)
    return pairs, sc, order


# ---------------------------------------------------------------- the engine
class Scene:
    """GPU scene: ISceneObject/BVHRT + MultiRenderer surface over the C ABI."""

    def __init__(self, device=0):
        self._ctx = C.c_void_p()
        _check(lib().lrt_create(C.byref(self._ctx), device), what="lrt_create (is a GPU visible?)")
        self.preset = Preset(RENDER_MODE_LAMBERT_NO_TEX, INTERSECT_ST, 0, 0, 0, 1, 1)

    def close(self):
        if self._ctx:
            lib().lrt_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, s):
        _check(s, self._ctx)

    def set_tuning(self, key, value):
        """Kernel choices that never change results ("variant", "block_warps")."""
        self._chk(lib().lrt_set_tuning(self._ctx, key.encode(), int(value)))

    def clear_geom(self):
        self._chk(lib().lrt_clear_geom(self._ctx))

    def add_sbs(self, header, nodes, values, values_f=None):
        nodes = np.ascontiguousarray(nodes, np.uint32).reshape(-1, 4)
        values = np.ascontiguousarray(values, np.uint32)
        vf = None if values_f is None else np.ascontiguousarray(values_f, np.float32)
        gid = C.c_uint32()
        self._chk(lib().lrt_add_sbs(self._ctx, C.byref(header), _ptr(nodes), nodes.shape[0], _ptr(values),
                                    values.size, _ptr(vf), 0 if vf is None else vf.size, C.byref(gid)))
        return gid.value

    def add_svs(self, nodes):
        nodes = np.ascontiguousarray(nodes, np.uint32).reshape(-1, 4)
        gid = C.c_uint32()
        self._chk(lib().lrt_add_svs(self._ctx, _ptr(nodes), nodes.shape[0], C.byref(gid)))
        return gid.value

    def add_triangles(self, vpos, indices):
        vpos = np.ascontiguousarray(vpos, np.float32)
        stride = vpos.shape[1] * 4
        idx = np.ascontiguousarray(indices, np.uint32).reshape(-1)
        gid = C.c_uint32()
        self._chk(lib().lrt_add_triangles(self._ctx, _ptr(vpos), vpos.shape[0], stride, _ptr(idx), idx.size,
                                          C.byref(gid)))
        return gid.value

    def refit_triangles(self, vpos):
        """Move the committed mesh's vertices (same count) and refit its BVH on the device."""
        vpos = np.ascontiguousarray(vpos, np.float32)
        self._chk(lib().lrt_refit_triangles(self._ctx, _ptr(vpos), vpos.shape[0], vpos.shape[1] * 4))

    def clear_scene(self):
        self._chk(lib().lrt_clear_scene(self._ctx))

    def add_instance(self, geom_id, matrix=None):
        m = np.ascontiguousarray(np.eye(4) if matrix is None else matrix, np.float32).reshape(16)
        iid = C.c_uint32()
        self._chk(lib().lrt_add_instance(self._ctx, geom_id, _ptr(m), C.byref(iid)))
        return iid.value

    def commit_scene(self):
        self._chk(lib().lrt_commit_scene(self._ctx))

    def update_instance(self, inst_id, matrix):
        """BVHRT::UpdateInstance: a new matrix for a committed instance."""
        m = np.ascontiguousarray(matrix, np.float32).reshape(16)
        self._chk(lib().lrt_update_instance(self._ctx, inst_id, _ptr(m)))

    def update_geom_triangles(self, geom_id, vpos, indices=None):
        """BVHRT::UpdateGeom_Triangles3f: new positions for the committed mesh (same connectivity)."""
        vpos = np.ascontiguousarray(vpos, np.float32)
        idx = None if indices is None else np.ascontiguousarray(indices, np.uint32).reshape(-1)
        self._chk(lib().lrt_update_geom_triangles(self._ctx, geom_id, _ptr(vpos), vpos.shape[0], _ptr(idx),
                                                  0 if idx is None else idx.size, vpos.shape[1] * 4))

    def add_aabb(self, boxes8, type_id=0):
        """BVHRT::AddGeom_AABB: refused (no intersector for custom boxes on this path)."""
        b = np.ascontiguousarray(boxes8, np.float32).reshape(-1, 8)
        gid = C.c_uint32()
        self._chk(lib().lrt_add_aabb(self._ctx, type_id, _ptr(b), b.shape[0], C.byref(gid)))
        return gid.value

    def set_seed(self, seed):
        """MultiRenderer::setSeed: seed of RAY_GEN_MODE_RANDOM's sub-pixel offsets."""
        self._chk(lib().lrt_set_seed(self._ctx, int(seed) & 0xFFFFFFFF))

    def set_bvh2(self, pairs):
        """The BVH2 (reference fat-pair layout, BVH_PAIR_DTYPE or 64-byte records) of the
        first-hit walk ("first_hit" tuning)."""
        p = np.ascontiguousarray(pairs)
        assert p.nbytes % 64 == 0
        self._chk(lib().lrt_set_bvh2(self._ctx, _ptr(p), p.nbytes // 64))

    def set_preset(self, render_mode=None, sdf_node_intersect=None, spp=None, representation_mode=None,
                   normal_mode=None, ray_gen_mode=None):
        p = self.preset
        if ray_gen_mode is not None:
            p.ray_gen_mode = ray_gen_mode
        if render_mode is not None:
            p.render_mode = render_mode
        if normal_mode is not None:
            p.normal_mode = normal_mode
        if sdf_node_intersect is not None:
            p.sdf_node_intersect = sdf_node_intersect
        if spp is not None:
            p.spp = spp
        if representation_mode is not None:
            p.representation_mode = representation_mode
        self._chk(lib().lrt_set_preset(self._ctx, C.byref(p)))

    # -- queries
    def query_rays(self, pos_near, dir_far):
        """Batched RayQuery_NearestHit on host arrays (n,4) -> structured hits."""
        pos = np.ascontiguousarray(pos_near, np.float32).reshape(-1, 4)
        dr = np.ascontiguousarray(dir_far, np.float32).reshape(-1, 4)
        out = np.zeros(pos.shape[0], HIT_DTYPE)
        self._chk(lib().lrt_query_rays(self._ctx, _ptr(pos), _ptr(dr), pos.shape[0], _ptr(out), 0, None))
        return out

    def query_rays_device(self, pos_ptr, dir_ptr, n, out_ptr, stream=0):
        self._chk(lib().lrt_query_rays(self._ctx, C.c_void_p(pos_ptr), C.c_void_p(dir_ptr), n,
                                       C.c_void_p(out_ptr), 1, C.c_void_p(stream)))

    def render_host(self, views, hits=True, rgba=False, rgba8=False):
        """views: list of (w, h, world_view, proj).  Returns dict of numpy arrays
        (flattened over views, row-major per view)."""
        va = make_views(views)
        npix = sum(int(w) * int(h) for w, h, _, _ in views)
        out = {}
        h16 = np.zeros(npix, HIT16_DTYPE) if hits else None
        col = np.zeros((npix, 4), np.float32) if rgba else None
        c8 = np.zeros(npix, np.uint32) if rgba8 else None
        self._chk(lib().lrt_render_host(self._ctx, C.cast(va, C.c_void_p), len(views), _ptr(h16), _ptr(col), _ptr(c8)))
        if hits:
            out["hits"] = h16
        if rgba:
            out["rgba"] = col
        if rgba8:
            out["rgba8"] = c8
        return out

    def render_device(self, view_array, n_views, hits_ptr=0, rgba_ptr=0, rgba8_ptr=0, stream=0):
        """Asynchronous render into device buffers (e.g. torch tensors' data_ptr())."""
        self._chk(lib().lrt_render(self._ctx, C.cast(view_array, C.c_void_p), n_views, C.c_void_p(hits_ptr or None),
                                   C.c_void_p(rgba_ptr or None), C.c_void_p(rgba8_ptr or None), C.c_void_p(stream or None)))

    def autotune(self, views, reps=3):
        """lrt_autotune: returns (best choice dict, list of all candidates tried)."""
        va = make_views(views)
        best = TuningChoice()
        allc = (TuningChoice * 64)()
        n = C.c_uint32()
        self._chk(lib().lrt_autotune(self._ctx, C.cast(va, C.c_void_p), len(views), reps, C.byref(best),
                                     C.cast(allc, C.c_void_p), 64, C.byref(n)))
        return best.as_dict(), [allc[i].as_dict() for i in range(n.value)]

    def graph_create(self, views, hits_ptr=0, rgba_ptr=0, rgba8_ptr=0):
        """lrt_render_graph_create over device output pointers; returns a handle."""
        va = make_views(views)
        g = C.c_void_p()
        self._chk(lib().lrt_render_graph_create(self._ctx, C.cast(va, C.c_void_p), len(views), C.c_void_p(hits_ptr or None),
                                                C.c_void_p(rgba_ptr or None), C.c_void_p(rgba8_ptr or None),
                                                C.byref(g)))
        return g

    def graph_launch(self, g, stream=0):
        self._chk(lib().lrt_render_graph_launch(self._ctx, g, C.c_void_p(stream or None)))

    def graph_set_views(self, g, views):
        va = make_views(views)
        self._chk(lib().lrt_render_graph_set_views(self._ctx, g, C.cast(va, C.c_void_p), len(views)))

    @staticmethod
    def graph_destroy(g):
        lib().lrt_render_graph_destroy(g)

    def last_launch_count(self):
        return lib().lrt_last_launch_count(self._ctx)

    def render_counters(self, views):
        va = make_views(views)
        out = np.zeros(4, np.uint64)
        self._chk(lib().lrt_render_counters(self._ctx, C.cast(va, C.c_void_p), len(views), _ptr(out)))
        return out

    def bvh2(self):
        """The committed BVH2 in the reference fat-pair layout (structured array)."""
        p, n = C.c_void_p(), C.c_uint32()
        self._chk(lib().lrt_get_bvh2(self._ctx, C.byref(p), C.byref(n)))
        buf = (C.c_uint8 * (n.value * 64)).from_address(p.value)
        return np.frombuffer(bytes(buf), BVH_PAIR_DTYPE).copy()
