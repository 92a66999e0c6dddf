"""ctypes binding of the differentiable-render part of the CPU oracle
(oracle/lrt_oracle_dr.c in oracle/_build/liblrt_oracle.so).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and bench.py's
CPU legs to verify and time against the GPU DR kernels.  The product never
imports this module.
"""
import ctypes as C

import numpy as np

from .oracle import SbsHeader, _p, _sdf_desc, lib, node_boxes, bvh2_build

VP = C.c_void_p

# RayQuery_NearestHitWithGrad record: 576 32-bit words (oracle/ref_driver.cpp)
HITDR = [("t", "<f4"), ("primId", "<u4"), ("instId", "<u4"), ("geomId", "<u4"), ("color", "<f4", (3,)),
         ("sdf", "<f4"), ("normal", "<f4", (3,)), ("check_vox_border", "<u4"), ("_pad", "<u4", (2,))]
PD_DIST = [("dDiffuse", "<f4", (3,)), ("index", "<u4"), ("dNorm", "<f4", (3,)), ("dDist", "<f4")]
RECORD_DTYPE = np.dtype([("hit", HITDR), ("missed_hit", HITDR), ("missed_indices", "<u4", (8,)),
                         ("missed_dSDF_dtheta", "<f4", (8,)), ("dc", [("index", "<u4"), ("value", "<f4")], (8,)),
                         ("dd", PD_DIST, (64,)), ("_tail", "<u4", (4,))])
assert RECORD_DTYPE.itemsize == 576 * 4

FLAG_DDIFFUSE_DCOLOR, FLAG_DDIFFUSE_DPOS, FLAG_DNORM_DPOS, FLAG_BORDER, FLAG_DDIST_DPOS = 1, 2, 4, 8, 16
RENDER_DIFFUSE, RENDER_LAMBERT, RENDER_MASK, RENDER_LINEAR_DEPTH, RENDER_NORMAL = 0, 1, 2, 3, 4
RECON_COLOR, RECON_GEOMETRY = 1, 2
LAYOUT_ID32F_IRGB32F, LAYOUT_ID32F_IRGB32F_IN = 4 << 24, 5 << 24


class DrScene_(C.Structure):
    _fields_ = [("hdr", SbsHeader), ("nodes", VP), ("n_nodes", C.c_uint32), ("values", VP), ("n_values", C.c_uint32),
                ("n_params", C.c_uint32), ("pairs", VP), ("n_pairs", C.c_uint32), ("inst_bmin", C.c_float * 3),
                ("inst_bmax", C.c_float * 3), ("inst_inv", C.c_float * 16), ("need_normal", C.c_int)]


class Light(C.Structure):
    _fields_ = [("type", C.c_uint32), ("dir", C.c_float * 3), ("color", C.c_float * 3)]


class DrPreset(C.Structure):
    _fields_ = [("render_mode", C.c_uint32), ("reconstruction_flags", C.c_uint32), ("input_type", C.c_uint32),
                ("loss_function", C.c_uint32), ("spp", C.c_uint32), ("border_spp", C.c_uint32),
                ("border_relax_eps", C.c_float), ("seed", C.c_uint32), ("n_lights", C.c_uint32),
                ("lights", Light * 4), ("lr", C.c_float), ("beta1", C.c_float), ("beta2", C.c_float),
                ("eps", C.c_float), ("accumulate_batch", C.c_uint32), ("reg_function", C.c_uint32),
                ("reg_lambda", C.c_float), ("reg_power", C.c_float), ("redistancing_enable", C.c_uint32),
                ("redistancing_interval", C.c_uint32), ("border_sampling", C.c_uint32),
                ("raycasting_mask", C.c_uint32)]


class DrView(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("proj_inv", C.c_float * 16),
                ("wv_inv", C.c_float * 16), ("proj", C.c_float * 16), ("world_view", C.c_float * 16),
                ("cast_mask", VP)]


class SvmLine(C.Structure):
    _fields_ = [("count", C.c_uint32), ("force", C.c_uint32), ("svm_spp", C.c_uint32), ("pad", C.c_uint32),
                ("p0", C.c_float * 2), ("r", C.c_float * 2), ("n", C.c_float * 2), ("radius", C.c_float),
                ("pdf", C.c_float)]


_bound = False


def _lib():
    global _bound
    L = lib()
    if not _bound:
        L.orc_dr_query.argtypes = [C.POINTER(DrScene_), VP, C.c_uint32, VP, VP, C.c_uint32, VP]
        L.orc_dr_render.restype = C.c_double
        L.orc_dr_render.argtypes = [C.POINTER(DrScene_), VP, C.POINTER(DrPreset), C.POINTER(DrView), VP, VP, VP, VP,
                                    VP, C.c_int]
        L.orc_dr_loss_f64.restype = C.c_double
        L.orc_dr_loss_f64.argtypes = [C.POINTER(DrScene_), VP, C.POINTER(DrPreset), C.POINTER(DrView), VP, VP]
        L.orc_dr_step.argtypes = [C.POINTER(DrScene_), VP, C.POINTER(DrPreset), VP, VP, C.c_uint32, C.c_uint32, VP,
                                  VP, VP, VP, C.c_int]
        L.orc_dr_adam.argtypes = [C.c_uint32, VP, VP, VP, C.c_uint32, C.c_float, C.c_float, C.c_float, C.c_float]
        L.orc_dr_regularize.argtypes = [C.POINTER(DrScene_), VP, C.POINTER(DrPreset), VP]
        L.orc_dr_redistance.argtypes = [VP, C.c_uint32, C.c_float, C.c_uint32]
        L.orc_dr_grid_resample.argtypes = [C.c_uint32, C.c_uint32, VP, C.c_uint32, VP]
        L.orc_dr_svm_fit.argtypes = [VP, C.c_uint32, VP]
        L.orc_dr_line_clip.restype = C.c_int
        L.orc_dr_line_clip.argtypes = [C.POINTER(C.c_float)] * 4
        L.orc_dr_svm_line.argtypes = [C.POINTER(DrScene_), VP, C.POINTER(DrPreset), C.POINTER(DrView), C.c_uint32,
                                      C.c_uint32, C.POINTER(SvmLine)]
        L.orc_dr_svm_sample.argtypes = [C.POINTER(SvmLine), C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, VP]
        L.orc_dr_grid_sbs.restype = C.c_uint32
        L.orc_dr_grid_sbs.argtypes = [C.c_uint32, C.c_uint32, C.c_void_p, VP, C.POINTER(SbsHeader), C.POINTER(VP),
                                      C.POINTER(VP), C.POINTER(C.c_uint32), C.POINTER(VP), C.POINTER(C.c_uint32)]
        _bound = True
    return L


def default_lights():
    """MultiRenderer's default lights (Renderer/eye_ray_host.cpp:40): a direct
    light along normalize(1,1,1) with colour 2/3 and an ambient 0.25."""
    d = np.ones(3, np.float32)
    d = d / np.sqrt(np.float32(3.0))
    return [(0, d, np.full(3, np.float32(2.0) / np.float32(3.0), np.float32)),
            (2, np.zeros(3, np.float32), np.full(3, 0.25, np.float32))]


def make_preset(render_mode=RENDER_LAMBERT, reconstruction=RECON_COLOR | RECON_GEOMETRY, input_type=0, loss=0,
                spp=1, border_spp=256, border_relax_eps=1e-3, seed=1, lights=None, lr=3e-3, beta1=0.9, beta2=0.999,
                eps=1e-8, accumulate_batch=0, reg_function=0, reg_lambda=0.25, reg_power=2.0,
                redistancing_enable=0, redistancing_interval=1, border_sampling=0, raycasting_mask=0):
    p = DrPreset()
    p.render_mode, p.reconstruction_flags, p.input_type, p.loss_function = render_mode, reconstruction, input_type, loss
    p.spp, p.border_spp, p.border_relax_eps, p.seed = spp, border_spp, border_relax_eps, seed
    lights = default_lights() if lights is None else lights
    p.n_lights = len(lights)
    for i, (t, d, c) in enumerate(lights):
        p.lights[i].type = t
        p.lights[i].dir[:] = [float(x) for x in np.asarray(d, np.float32)]
        p.lights[i].color[:] = [float(x) for x in np.asarray(c, np.float32)]
    p.lr, p.beta1, p.beta2, p.eps, p.accumulate_batch = lr, beta1, beta2, eps, accumulate_batch
    p.reg_function, p.reg_lambda, p.reg_power = reg_function, reg_lambda, reg_power
    p.redistancing_enable, p.redistancing_interval = redistancing_enable, redistancing_interval
    p.border_sampling, p.raycasting_mask = border_sampling, raycasting_mask
    return p


def svm_fit(rows):
    """SVM_fit on rows (n, 3) = (x, y, 1) * label; returns (a, b, c, error rate)."""
    X = np.ascontiguousarray(rows, np.float32).copy()
    W = np.zeros(4, np.float32)
    _lib().orc_dr_svm_fit(_p(X), X.shape[0], _p(W))
    return W


def line_clip(x0, y0, x1, y1):
    """CohenSutherlandLineClip against [0,1]^2: (accepted, x0, y0, x1, y1)."""
    v = [C.c_float(x0), C.c_float(y0), C.c_float(x1), C.c_float(y1)]
    ok = _lib().orc_dr_line_clip(*[C.byref(a) for a in v])
    return bool(ok), v[0].value, v[1].value, v[2].value, v[3].value


def make_view(width, height, world_view, proj, inverse4x4):
    v = DrView()
    v.width, v.height = width, height
    wv = np.asarray(world_view, np.float32).reshape(16)
    pj = np.asarray(proj, np.float32).reshape(16)
    v.proj_inv[:] = np.asarray(inverse4x4(pj), np.float32).reshape(16).tolist()
    v.wv_inv[:] = np.asarray(inverse4x4(wv), np.float32).reshape(16).tolist()
    v.proj[:] = pj.tolist()
    v.world_view[:] = wv.tolist()
    return v


def grid_sbs(brick_count, brick_size, spheres=None, boxes=None, k=0.0, color=None):
    """create_grid_sbs + neighbour table; returns (header, nodes[n,4], values, params)."""
    d, keep = _sdf_desc(spheres, boxes, k)
    L = _lib()
    hdr = SbsHeader()
    pn, pv, pp = VP(), VP(), VP()
    nv, npar = C.c_uint32(), C.c_uint32()
    col = None if color is None else np.ascontiguousarray(color, np.float32)
    n = L.orc_dr_grid_sbs(brick_count, brick_size, C.cast(C.pointer(d), VP), _p(col), C.byref(hdr), C.byref(pn),
                          C.byref(pv), C.byref(nv), C.byref(pp), C.byref(npar))
    nodes = np.ctypeslib.as_array(C.cast(pn, C.POINTER(C.c_uint32)), (n * 4,)).copy().reshape(-1, 4)
    values = np.ctypeslib.as_array(C.cast(pv, C.POINTER(C.c_uint32)), (nv.value,)).copy()
    params = np.ctypeslib.as_array(C.cast(pp, C.POINTER(C.c_float)), (npar.value,)).copy()
    for q in (pn, pv, pp):
        L.orc_free(q)
    return hdr, nodes, values, params


class DrScene:
    """An indexed SBS (ID32F_IRGB32F or _IN layout) with its BVH2 and one identity instance."""

    def __init__(self, hdr, nodes, values, n_params, pairs=None, need_normal=True):
        s = DrScene_()
        nodes = np.ascontiguousarray(nodes, np.uint32).reshape(-1, 4)
        values = np.ascontiguousarray(values, np.uint32)
        if pairs is None:
            pairs = bvh2_build(node_boxes(nodes), 1)[0]
        pairs = np.ascontiguousarray(pairs)
        self.keep = [nodes, values, pairs]
        s.hdr = SbsHeader(hdr.brick_size, hdr.brick_pad, hdr.bytes_per_value, hdr.aux_data)
        s.nodes, s.n_nodes, s.values, s.n_values = _p(nodes), nodes.shape[0], _p(values), values.size
        s.n_params = n_params
        s.pairs, s.n_pairs = _p(pairs), pairs.nbytes // 64
        s.inst_bmin[:] = [-1.0, -1.0, -1.0]
        s.inst_bmax[:] = [1.0, 1.0, 1.0]
        s.inst_inv[:] = np.eye(4, dtype=np.float32).reshape(16).tolist()
        s.need_normal = 1 if need_normal else 0
        self.s = s
        self.pairs = pairs

    def query(self, params, flags, pos_near, dir_far):
        P = np.ascontiguousarray(params, np.float32)
        pos = np.ascontiguousarray(pos_near, np.float32).reshape(-1, 4)
        dr = np.ascontiguousarray(dir_far, np.float32).reshape(-1, 4)
        out = np.zeros(pos.shape[0], RECORD_DTYPE)
        _lib().orc_dr_query(C.byref(self.s), _p(P), flags, _p(pos), _p(dr), pos.shape[0], _p(out))
        return out

    def render(self, params, preset, view, image_ref, threads=0, mask=None):
        """mask: the view's W*H uint8 ray-casting mask, read and rewritten in place
        (preset.raycasting_mask on)."""
        view.cast_mask = None if mask is None else _p(mask)
        P = np.ascontiguousarray(params, np.float32)
        n = view.width * view.height
        ref = np.ascontiguousarray(image_ref, np.float32).reshape(n, 4)
        img = np.zeros((n, 4), np.float32)
        dep = np.zeros(n, np.float32)
        grad = np.zeros(P.size, np.float32)
        border = np.zeros(n, np.uint8)
        loss = _lib().orc_dr_render(C.byref(self.s), _p(P), C.byref(preset), C.byref(view), _p(ref), _p(img), _p(dep),
                                    _p(grad), _p(border), threads)
        return dict(loss=loss, image=img, depth=dep, grad=grad, border=border.astype(bool))

    def loss_f64(self, params_d, preset, view, image_ref):
        P = np.ascontiguousarray(params_d, np.float64)
        n = view.width * view.height
        ref = np.ascontiguousarray(image_ref, np.float32).reshape(n, 4)
        hc = np.zeros(n, np.uint8)
        loss = _lib().orc_dr_loss_f64(C.byref(self.s), _p(P), C.byref(preset), C.byref(view), _p(ref), _p(hc))
        return loss, hc

    def regularize(self, params, preset):
        """Regularization's gradient alone (diff_render/MultiRendererDR.cpp:1933-2055)."""
        params = np.ascontiguousarray(params, np.float32)
        g = np.zeros(params.size, np.float32)
        _lib().orc_dr_regularize(C.byref(self.s), _p(params), C.byref(preset), _p(g))
        return g

    def step(self, params, preset, views, images, it, adam_state, threads=0, masks=None):
        """One OptimizeFixedStructure iteration; params and adam_state are updated in
        place, and so are the views' uint8 ray-casting masks when given."""
        assert params.dtype == np.float32 and params.flags.c_contiguous
        assert adam_state.dtype == np.float32 and adam_state.size == 2 * params.size
        nv = len(views)
        for k, v in enumerate(views):
            v.cast_mask = None if masks is None else _p(masks[k])
        va = (DrView * nv)(*views)
        imgs = np.ascontiguousarray(np.concatenate([np.asarray(i, np.float32).reshape(-1, 4) for i in images]))
        grad = np.zeros(params.size, np.float32)
        losses = np.zeros(nv, np.float64)
        out_imgs = np.zeros_like(imgs)
        _lib().orc_dr_step(C.byref(self.s), _p(params), C.byref(preset), C.cast(va, VP), _p(imgs), nv, it,
                           _p(adam_state), _p(grad), _p(losses), _p(out_imgs), threads)
        return dict(grad=grad, losses=losses, images=out_imgs)

    def svm_line(self, params, preset, view, x, y):
        """The SVM stage of CastBorderRaySVM for pixel (x, y): an SvmLine."""
        P = np.ascontiguousarray(params, np.float32)
        L = SvmLine()
        _lib().orc_dr_svm_line(C.byref(self.s), _p(P), C.byref(preset), C.byref(view), x, y, C.byref(L))
        return L


def adam(it, g, x, state, lr, b1=0.9, b2=0.999, eps=1e-8):
    g = np.ascontiguousarray(g, np.float32)
    _lib().orc_dr_adam(it, _p(g), _p(x), _p(state), x.size, lr, b1, b2, eps)


def redistance(dist, n, h, iters):
    """Redistance (diff_render/MultiRendererDR.cpp:2122-2330) of a dense n^3 grid; returns a copy."""
    d = np.ascontiguousarray(dist, np.float32).copy()
    _lib().orc_dr_redistance(_p(d), n, h, iters)
    return d


def grid_resample(gs, bs, old_params=None, old_bs=0):
    """OptimizeGrid's grid parameters: the starting grid (old_params None) or the
    distances of old_params resampled into bricks of bs."""
    n = (gs * bs + 1) ** 3 + 3 * (gs + 1) ** 3
    out = np.zeros(n, np.float32)
    op = None if old_params is None else np.ascontiguousarray(old_params, np.float32)
    _lib().orc_dr_grid_resample(gs, bs, _p(op), old_bs, _p(out))
    return out

