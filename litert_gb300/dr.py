"""Python host mirror of the differentiable-render C ABI (include/lrt_dr.h).

``MultiRendererDR`` follows dr::MultiRendererDR (diff_render/MultiRendererDR.h:71-155):
``SetLights``, ``SetReference``, ``OptimizeFixedStructure`` (which updates the
indexed SBS's ``values_f`` in place as the reference does at
diff_render/MultiRendererDR.cpp:575), ``getLastImage`` and
``getLastdLoss_dS``, plus the per-view ``render_grad`` / ``step`` building
blocks.  Everything runs in the compiled engine on the GPU; there is no CPU
fallback.
"""
import ctypes as C

import numpy as np

from . import lrt

RENDER_DIFFUSE, RENDER_LAMBERT, RENDER_MASK, RENDER_LINEAR_DEPTH, RENDER_NORMAL = 0, 1, 2, 3, 4
RECON_COLOR, RECON_GEOMETRY = 1, 2
LIGHT_DIRECT, LIGHT_AMBIENT = 0, 2
GET_PARAMS, GET_GRAD, GET_IMAGE, GET_DEPTH, GET_BORDER, GET_ADAM, GET_CAST_MASK = 0, 1, 2, 3, 4, 5, 6


class Light(C.Structure):
    _fields_ = [("type", C.c_uint32), ("dir", C.c_float * 3), ("color", C.c_float * 3)]


class DrPreset(C.Structure):
    _fields_ = [("render_mode", C.c_uint32), ("reconstruction_flags", C.c_uint32), ("input_type", C.c_uint32),
                ("loss_function", C.c_uint32), ("spp", C.c_uint32), ("border_spp", C.c_uint32),
                ("border_relax_eps", C.c_float), ("seed", C.c_uint32), ("n_lights", C.c_uint32),
                ("lights", Light * 4), ("opt_lr", C.c_float), ("opt_beta_1", C.c_float), ("opt_beta_2", C.c_float),
                ("opt_eps", C.c_float), ("accumulate_batch", C.c_uint32), ("warp_aggregate", C.c_uint32),
                ("reg_function", C.c_uint32), ("reg_lambda", C.c_float), ("reg_power", C.c_float),
                ("redistancing_enable", C.c_uint32), ("redistancing_interval", C.c_uint32),
                ("border_sampling", C.c_uint32), ("raycasting_mask", C.c_uint32)]


_bound = False


def _lib():
    global _bound
    L = lrt.lib()
    if not _bound:
        P, U32, I, VP = C.c_void_p, C.c_uint32, C.c_int, C.c_void_p
        sig = {
            "lrt_dr_default_preset": (None, [C.POINTER(DrPreset)]),
            "lrt_dr_set_scene": (I, [P, C.POINTER(lrt.SbsHeader), VP, U32, VP, C.c_uint64, VP, U32, VP, U32]),
            "lrt_dr_get_bvh2": (I, [P, C.POINTER(VP), C.POINTER(U32)]),
            "lrt_dr_set_reference": (I, [P, U32, VP, VP]),
            "lrt_dr_set_preset": (I, [P, C.POINTER(DrPreset)]),
            "lrt_dr_set_params": (I, [P, VP, U32]),
            "lrt_dr_render_grad": (I, [P, U32, C.POINTER(C.c_double)]),
            "lrt_dr_step": (I, [P, U32, VP]),
            "lrt_dr_optimize": (I, [P, U32, U32, VP]),
            "lrt_dr_get": (I, [P, U32, U32, VP, C.c_uint64]),
            "lrt_dr_last_launch_count": (U32, [P]),
            "lrt_dr_query_rays": (I, [P, U32, VP, VP, U32, VP]),
            "lrt_dr_grid_sbs": (I, [U32, U32, C.POINTER(lrt.SdfDesc), VP, C.POINTER(lrt.SbsHeader), C.POINTER(VP),
                                    C.POINTER(U32), C.POINTER(VP), C.POINTER(C.c_uint64), C.POINTER(VP),
                                    C.POINTER(U32)]),
            "lrt_dr_grid_resample": (I, [U32, U32, VP, U32, C.POINTER(lrt.SbsHeader), C.POINTER(VP), C.POINTER(U32),
                                         C.POINTER(VP), C.POINTER(C.c_uint64), C.POINTER(VP), C.POINTER(U32)]),
            "lrt_dr_optimize_grid": (I, [P, U32, U32, VP, VP, VP, U32, C.POINTER(lrt.SbsHeader), C.POINTER(VP),
                                         C.POINTER(U32), C.POINTER(VP), C.POINTER(C.c_uint64), C.POINTER(VP),
                                         C.POINTER(U32), VP]),
            "lrt_dr_preprocess_reference": (I, [U32, VP, VP, U32, U32, VP, VP]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _bound = True
    return L


def default_preset(**kw):
    """getDefaultPresetDR with a colour+geometry Lambert reconstruction; keyword
    arguments override fields (lights: list of (type, dir, color))."""
    p = DrPreset()
    _lib().lrt_dr_default_preset(C.byref(p))
    lights = kw.pop("lights", None)
    for k, v in kw.items():
        if not hasattr(p, k):
            raise KeyError(k)
        setattr(p, k, v)
    if lights is not None:
        p.n_lights = len(lights)
        for i, (t, d, c) in enumerate(lights):
            p.lights[i].type = t
            p.lights[i].dir[:] = [float(x) for x in np.asarray(d, np.float32)]
            p.lights[i].color[:] = [float(x) for x in np.asarray(c, np.float32)]
    return p


def _take_grid(L, hdr, pn, nn, pv, nv, pp, npar):
    try:
        nodes = np.ctypeslib.as_array(C.cast(pn, C.POINTER(C.c_uint32)), (nn.value * 4,)).copy().reshape(-1, 4)
        values = np.ctypeslib.as_array(C.cast(pv, C.POINTER(C.c_uint32)), (nv.value,)).copy()
        params = np.ctypeslib.as_array(C.cast(pp, C.POINTER(C.c_float)), (npar.value,)).copy()
    finally:
        for q in (pn, pv, pp):
            L.lrt_free(q)
    return hdr, nodes, values, params


def preprocess_reference(views, images, width, height):
    """PreprocessRefImages: the reference images (list of HxWx4 float) resampled to
    width x height; returns (views with the new size, list of images)."""
    from .lrt import make_views
    va = make_views(views)
    imgs = np.ascontiguousarray(np.concatenate([np.asarray(i, np.float32).reshape(-1, 4) for i in images]))
    out_v = (lrt.View * len(views))()
    out = np.zeros((len(views) * width * height, 4), np.float32)
    lrt._check(_lib().lrt_dr_preprocess_reference(len(views), C.cast(va, C.c_void_p), lrt._ptr(imgs), width, height,
                                                  C.cast(out_v, C.c_void_p), lrt._ptr(out)),
               what="lrt_dr_preprocess_reference")
    return out_v, [out[k * width * height:(k + 1) * width * height].reshape(height, width, 4)
                   for k in range(len(views))]


def grid_resample(brick_count, brick_size, old_params=None, old_brick_size=0):
    """create_grid_sbs as OptimizeGrid calls it: the starting grid (old_params None)
    or old_params's distances resampled into bricks of brick_size; gradient colours."""
    L = _lib()
    hdr = lrt.SbsHeader()
    pn, pv, pp = C.c_void_p(), C.c_void_p(), C.c_void_p()
    nn, npar, nv = C.c_uint32(), C.c_uint32(), C.c_uint64()
    op = None if old_params is None else np.ascontiguousarray(old_params, np.float32)
    lrt._check(L.lrt_dr_grid_resample(brick_count, brick_size, lrt._ptr(op), old_brick_size, C.byref(hdr),
                                      C.byref(pn), C.byref(nn), C.byref(pv), C.byref(nv), C.byref(pp),
                                      C.byref(npar)), what="lrt_dr_grid_resample")
    return _take_grid(L, hdr, pn, nn, pv, nv, pp, npar)


def grid_sbs(brick_count, brick_size, sdf, color=None):
    """create_grid_sbs + SBS_ind_to_SBS_ind_with_neighbors on the host:
    returns (header, nodes (n,4) u32, values u32, params f32)."""
    L = _lib()
    hdr = lrt.SbsHeader()
    pn, pv, pp = C.c_void_p(), C.c_void_p(), C.c_void_p()
    nn, npar, nv = C.c_uint32(), C.c_uint32(), C.c_uint64()
    col = None if color is None else np.ascontiguousarray(color, np.float32)
    lrt._check(L.lrt_dr_grid_sbs(brick_count, brick_size, C.byref(sdf.desc()), lrt._ptr(col), C.byref(hdr),
                                 C.byref(pn), C.byref(nn), C.byref(pv), C.byref(nv), C.byref(pp), C.byref(npar)),
               what="lrt_dr_grid_sbs")
    try:
        nodes = np.ctypeslib.as_array(C.cast(pn, C.POINTER(C.c_uint32)), (nn.value * 4,)).copy().reshape(-1, 4)
        values = np.ctypeslib.as_array(C.cast(pv, C.POINTER(C.c_uint32)), (nv.value,)).copy()
        params = np.ctypeslib.as_array(C.cast(pp, C.POINTER(C.c_float)), (npar.value,)).copy()
    finally:
        for q in (pn, pv, pp):
            L.lrt_free(q)
    return hdr, nodes, values, params


class MultiRendererDR:
    """GPU dr::MultiRendererDR over one context of the engine."""

    def __init__(self, device=0):
        self._ctx = C.c_void_p()
        lrt._check(lrt.lib().lrt_create(C.byref(self._ctx), device), what="lrt_create")
        self.preset = default_preset()
        self.n_params = 0
        self.views = []
        self._keep = []

    def close(self):
        if self._ctx:
            lrt.lib().lrt_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, s):
        if s != 0:
            raise lrt.LrtError(s, lrt.lib().lrt_last_error(self._ctx).decode())

    def set_tuning(self, key, value):
        """lrt_set_tuning on this context ("bvh_builder" 1: SetScene builds the BVH on the device)."""
        self._chk(lrt.lib().lrt_set_tuning(self._ctx, key.encode(), int(value)))

    # ---- scene / reference / preset
    def SetScene(self, hdr, nodes, values, params, pairs=None):
        nodes = np.ascontiguousarray(nodes, np.uint32).reshape(-1, 4)
        values = np.ascontiguousarray(values, np.uint32)
        params = np.ascontiguousarray(params, np.float32)
        pr = None if pairs is None else np.ascontiguousarray(pairs)
        self._chk(_lib().lrt_dr_set_scene(self._ctx, C.byref(hdr), lrt._ptr(nodes), nodes.shape[0], lrt._ptr(values),
                                          values.size, lrt._ptr(params), params.size, lrt._ptr(pr),
                                          0 if pr is None else pr.nbytes // 64))
        self.n_params = params.size

    def bvh2(self):
        p, n = C.c_void_p(), C.c_uint32()
        self._chk(_lib().lrt_dr_get_bvh2(self._ctx, C.byref(p), C.byref(n)))
        return np.ctypeslib.as_array(C.cast(p, C.POINTER(C.c_uint8)), (n.value * 64,)).copy()

    def SetReference(self, images, worldView, proj):
        views = [(np.asarray(im).shape[1], np.asarray(im).shape[0], wv, pj) for im, wv, pj in zip(images, worldView, proj)]
        self.views = views
        arr = lrt.make_views(views)
        imgs = np.ascontiguousarray(np.concatenate([np.asarray(im, np.float32).reshape(-1, 4) for im in images]))
        self._keep = [arr, imgs]
        self._chk(_lib().lrt_dr_set_reference(self._ctx, len(views), C.cast(arr, C.c_void_p), lrt._ptr(imgs)))

    def SetPreset(self, preset):
        self.preset = preset
        self._chk(_lib().lrt_dr_set_preset(self._ctx, C.byref(preset)))

    def SetLights(self, lights):
        p = DrPreset.from_buffer_copy(self.preset)
        p.n_lights = len(lights)
        for i, (t, d, c) in enumerate(lights):
            p.lights[i].type = t
            p.lights[i].dir[:] = [float(x) for x in np.asarray(d, np.float32)]
            p.lights[i].color[:] = [float(x) for x in np.asarray(c, np.float32)]
        self.SetPreset(p)

    def set_params(self, params):
        params = np.ascontiguousarray(params, np.float32)
        self._chk(_lib().lrt_dr_set_params(self._ctx, lrt._ptr(params), params.size))

    # ---- gradients and optimisation
    def render_grad(self, view):
        """RenderDR of one view: returns (loss, gradient)."""
        loss = C.c_double()
        self._chk(_lib().lrt_dr_render_grad(self._ctx, view, C.byref(loss)))
        return loss.value, self.get(GET_GRAD)

    def step(self, it, want_losses=True):
        losses = np.zeros(len(self.views), np.float64) if want_losses else None
        self._chk(_lib().lrt_dr_step(self._ctx, it, lrt._ptr(losses)))
        return losses

    def OptimizeFixedStructure(self, preset, sbs, iterations, first_iter=0):
        """sbs = [hdr, nodes, values, params]; params (sbs[3]) is updated in place."""
        self.SetPreset(preset)
        self.SetScene(*sbs[:4])
        last = np.zeros(len(self.views), np.float64)
        self._chk(_lib().lrt_dr_optimize(self._ctx, first_iter, iterations, lrt._ptr(last)))
        sbs[3][:] = self.get(GET_PARAMS)
        return last

    def OptimizeGrid(self, start_grid_size, no_last_step_resize, presets, iterations, render_sizes=None):
        """MultiRendererDR::OptimizeGrid on the reference set by SetReference (each
        stage at render_sizes[i] = (width, height), or as given): returns (final grid
        [hdr, nodes, values, params], last step's per-view losses)."""
        L = _lib()
        pa = (DrPreset * len(presets))(*presets)
        it = np.ascontiguousarray(iterations, np.uint32)
        rs = None if render_sizes is None else np.ascontiguousarray(render_sizes, np.uint32).reshape(-1)
        hdr = lrt.SbsHeader()
        pn, pv, pp = C.c_void_p(), C.c_void_p(), C.c_void_p()
        nn, npar, nv = C.c_uint32(), C.c_uint32(), C.c_uint64()
        last = np.zeros(len(self.views), np.float64)
        self._chk(L.lrt_dr_optimize_grid(self._ctx, start_grid_size, int(bool(no_last_step_resize)),
                                         C.cast(pa, C.c_void_p), lrt._ptr(it), lrt._ptr(rs), len(presets), C.byref(hdr),
                                         C.byref(pn), C.byref(nn), C.byref(pv), C.byref(nv), C.byref(pp),
                                         C.byref(npar), lrt._ptr(last)))
        grid = list(_take_grid(L, hdr, pn, nn, pv, nv, pp, npar))
        self.n_params = grid[3].size
        return grid, last

    def get(self, what, view=0):
        if what in (GET_PARAMS, GET_GRAD):
            out = np.zeros(self.n_params, np.float32)
        elif what == GET_ADAM:
            out = np.zeros(2 * self.n_params, np.float32)
        else:
            w, h = self.views[view][0], self.views[view][1]
            out = {GET_IMAGE: np.zeros((h * w, 4), np.float32), GET_DEPTH: np.zeros(h * w, np.float32),
                   GET_BORDER: np.zeros(h * w, np.uint8), GET_CAST_MASK: np.zeros(h * w, np.uint8)}[what]
        self._chk(_lib().lrt_dr_get(self._ctx, what, view, lrt._ptr(out), out.nbytes))
        return out

    def getLastImage(self, view):
        w, h = self.views[view][0], self.views[view][1]
        return self.get(GET_IMAGE, view).reshape(h, w, 4)

    def getLastdLoss_dS(self):
        return self.get(GET_GRAD)

    def query_rays(self, flags, pos_near, dir_far):
        """RayQuery_NearestHitWithGrad on a ray batch: (n, 32) uint32 records (see lrt_dr.h)."""
        pos = np.ascontiguousarray(pos_near, np.float32).reshape(-1, 4)
        d = np.ascontiguousarray(dir_far, np.float32).reshape(-1, 4)
        out = np.zeros((pos.shape[0], 32), np.uint32)
        self._chk(_lib().lrt_dr_query_rays(self._ctx, flags, lrt._ptr(pos), lrt._ptr(d), pos.shape[0], lrt._ptr(out)))
        return out

    def last_launch_count(self):
        return _lib().lrt_dr_last_launch_count(self._ctx)
