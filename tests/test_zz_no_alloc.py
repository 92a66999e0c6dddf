"""GPU: the rendering entry point that allocates nothing (lrt_render_noalloc).

It serves callers that must not allocate device memory while rendering (an
application pool allocator that owns the GPU's memory, a real-time loop that
cannot afford cudaMalloc's synchronisation).  Its scratch lives in a
file-scope device array shared by all calls, so the test checks its output
against the allocating entry point on two calls in a row -- the second call
must not see stale state from the first -- and that more views than the array
holds are rejected.  This file sorts last so that, when it fails, a run that
stops at the first failure has already run every other test; it also passes
on its own in a fresh process (the first call sets the array up).
"""
import ctypes as C

import numpy as np
import pytest

from litert_gb300 import lrt, scenes

pytestmark = pytest.mark.gpu


def _scene():
    p = scenes.union_params()
    h, n, v = lrt.sbs_from_sdf(lrt.Sdf(**p), 5, 4)
    s = lrt.Scene(0)
    g = s.add_sbs(h, n, v)
    s.add_instance(g)
    s.commit_scene()
    s.set_preset(render_mode=lrt.RENDER_MODE_LAMBERT_NO_TEX, sdf_node_intersect=lrt.INTERSECT_NEWTON)
    return s


def _bits(a):
    a = np.ascontiguousarray(a, np.float32)
    b = a.view(np.uint32).copy()
    b[np.isnan(a)] = 0x7FC00000
    return b


def test_render_noalloc_matches_render_on_two_calls():
    import torch

    s = _scene()
    try:
        views = scenes.union_views(n_views=3, lo=96, hi=160)
        npix = sum(w * h for w, h, _, _ in views)
        ref = s.render_host(views, hits=True, rgba=True)          # the allocating entry point
        va = lrt.make_views(views)
        dev = torch.device("cuda", 0)
        hits = torch.empty(npix * 4, dtype=torch.float32, device=dev)
        rgba = torch.empty(npix * 4, dtype=torch.float32, device=dev)
        stream = torch.cuda.current_stream(dev)
        for call in range(2):
            hits.fill_(float("nan"))
            rgba.fill_(-1.0)
            st = lrt.lib().lrt_render_noalloc(s._ctx, C.cast(va, C.c_void_p), len(views),
                                              C.c_void_p(hits.data_ptr()), C.c_void_p(rgba.data_ptr()), None,
                                              C.c_void_p(stream.cuda_stream))
            assert st == 0, f"call {call}: status {st}"
            torch.cuda.synchronize(dev)
            got_hits = hits.cpu().numpy().view(lrt.HIT16_DTYPE)
            got_rgba = rgba.cpu().numpy().reshape(-1, 4)
            assert (got_hits["primId"] != lrt.MISS).sum() > 0
            # same kernels as lrt_render: bit-identical records (NaN == NaN)
            assert np.array_equal(got_hits["primId"], ref["hits"]["primId"]), f"call {call}"
            for f in ("t", "nx", "ny"):
                assert np.array_equal(_bits(got_hits[f]), _bits(ref["hits"][f])), f"call {call}: {f}"
            assert np.array_equal(_bits(got_rgba), _bits(ref["rgba"])), f"call {call}: rgba"
        # more views than the scratch array holds is rejected, nothing launched
        many = lrt.make_views([scenes.sphere_view(8, 8)] * 65)
        st = lrt.lib().lrt_render_noalloc(s._ctx, C.cast(many, C.c_void_p), 65, C.c_void_p(hits.data_ptr()),
                                          None, None, None)
        assert st == 1   # LRT_ERR_INVALID
    finally:
        s.close()


def test_render_noalloc_first_hit_after_the_tree_is_on_the_device():
    """With the "first_hit" tuning key the entry point renders the reference's
    first-hit walk, as lrt_render does.  That walk's tree is put on the device
    by the first allocating call after a commit; before it, the entry point
    refuses (LRT_ERR_STATE) instead of allocating."""
    import torch

    s = _scene()
    try:
        s.set_tuning("first_hit", 1)
        views = scenes.union_views(n_views=2, lo=96, hi=128)
        npix = sum(w * h for w, h, _, _ in views)
        va = lrt.make_views(views)
        dev = torch.device("cuda", 0)
        hits = torch.empty(npix * 4, dtype=torch.float32, device=dev)
        stream = torch.cuda.current_stream(dev)

        def call():
            return lrt.lib().lrt_render_noalloc(s._ctx, C.cast(va, C.c_void_p), len(views),
                                                C.c_void_p(hits.data_ptr()), None, None,
                                                C.c_void_p(stream.cuda_stream))

        assert call() == 7   # LRT_ERR_STATE: the walk's tree is not on the device yet
        ref = s.render_host(views, hits=True)["hits"]   # lrt_render uploads it
        for k in range(2):
            hits.fill_(float("nan"))
            assert call() == 0, f"call {k}"
            torch.cuda.synchronize(dev)
            got = hits.cpu().numpy().view(lrt.HIT16_DTYPE)
            assert (got["primId"] != lrt.MISS).sum() > 0
            assert np.array_equal(got["primId"], ref["primId"]), f"call {k}"
            for f in ("t", "nx", "ny"):
                assert np.array_equal(_bits(got[f]), _bits(ref[f])), f"call {k}: {f}"
    finally:
        s.close()
