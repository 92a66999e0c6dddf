"""GPU: failure paths, made on the host or with a bounded wait -- no GPU fault.

* The tcgen05 network engine's per-layer completion wait is bounded ("tc_wait"
  polls).  With 0 polls every block gives up at its first wait: the call returns
  LRT_ERR_TIMEOUT after the blocks have drained the tensor-core work they issued
  and freed their tensor memory, and the next call, with the default limit, runs
  normally and matches the warp-level engine.
* Host-side fault injection (LRT_INJECT_FAULT): a failed device allocation, a
  failed scene upload and a failed graph instantiation each return a clean
  status (LRT_ERR_OOM / LRT_ERR_CUDA) and leave the context usable: once the
  injection is lifted the same calls succeed and render what an untouched
  context renders.
"""
import os

import numpy as np
import pytest

from litert_gb300 import lrt, proposal as pp, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture
def inject():
    def set_site(site):
        if site is None:
            os.environ.pop("LRT_INJECT_FAULT", None)
        else:
            os.environ["LRT_INJECT_FAULT"] = site
    yield set_site
    os.environ.pop("LRT_INJECT_FAULT", None)


def _sbs():
    return lrt.sbs_from_sdf(lrt.Sdf(**scenes.union_params()), 4, 4)


def test_tcgen05_wait_timeout_then_recovers():
    h, n, v = _sbs()
    s = lrt.Scene(0)
    try:
        s.add_instance(s.add_sbs(h, n, v))
        s.commit_scene()
        rng = np.random.default_rng(2)
        x = rng.uniform(0, 1, (5000, 16)).astype(np.float32)
        t = rng.uniform(0, 1, 5000).astype(np.float32)
        pp.set_weights(s, pp.init_weights(7))
        pp.set_triples(s, x, t)
        s.set_tuning("tc_wait", 0)
        with pytest.raises(lrt.LrtError) as e:
            pp.infer(s, 0, 5000, engine=pp.ENGINE_TCGEN05)
        assert e.value.status == 5   # LRT_ERR_TIMEOUT
        s.set_tuning("tc_wait", 1 << 20)
        y_tc = pp.infer(s, 0, 5000, engine=pp.ENGINE_TCGEN05)
        y_mma = pp.infer(s, 0, 5000, engine=pp.ENGINE_MMA)
        assert np.abs(y_tc - y_mma).max() <= 1e-3 * (np.abs(y_mma).max() + 1e-6)
    finally:
        s.close()


@pytest.mark.parametrize("site,status", [("alloc", 2), ("upload", 3)])
def test_commit_fault_is_clean(inject, site, status):
    h, n, v = _sbs()
    view = scenes.union_views(n_views=1, lo=64, hi=80)[0]
    ref = lrt.Scene(0)
    ref.add_instance(ref.add_sbs(h, n, v))
    ref.commit_scene()
    ref.set_preset(render_mode=lrt.RENDER_MODE_NORMAL, sdf_node_intersect=lrt.INTERSECT_NEWTON)
    want = ref.render_host([view], hits=True)["hits"]
    ref.close()
    s = lrt.Scene(0)
    try:
        s.add_instance(s.add_sbs(h, n, v))
        inject(site)
        with pytest.raises(lrt.LrtError) as e:
            s.commit_scene()
        assert e.value.status == status
        inject(None)
        with pytest.raises(lrt.LrtError) as e:   # nothing committed: rendering is refused, not attempted
            s.render_host([view], hits=True)
        assert e.value.status == 7
        s.commit_scene()
        s.set_preset(render_mode=lrt.RENDER_MODE_NORMAL, sdf_node_intersect=lrt.INTERSECT_NEWTON)
        got = s.render_host([view], hits=True)["hits"]
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    finally:
        s.close()


def test_graph_instantiation_fault_is_clean(inject):
    import ctypes as C
    import torch
    h, n, v = _sbs()
    views = scenes.union_views(n_views=2, lo=64, hi=80)
    npix = sum(w * hh for w, hh, _, _ in views)
    s = lrt.Scene(0)
    try:
        s.add_instance(s.add_sbs(h, n, v))
        s.commit_scene()
        s.set_preset(render_mode=lrt.RENDER_MODE_NORMAL, sdf_node_intersect=lrt.INTERSECT_NEWTON)
        want = s.render_host(views, hits=True)["hits"]
        out = torch.zeros(npix * 4, dtype=torch.float32, device="cuda:0")
        inject("graph")
        g = C.c_void_p()
        va = lrt.make_views(views)
        st = lrt.lib().lrt_render_graph_create(s._ctx, C.cast(va, C.c_void_p), len(views), C.c_void_p(out.data_ptr()),
                                               None, None, C.byref(g))
        assert st == 3 and not g.value
        inject(None)
        g = s.graph_create(views, hits_ptr=out.data_ptr())
        s.graph_launch(g)
        torch.cuda.synchronize()
        lrt.Scene.graph_destroy(g)
        got = out.cpu().numpy().view(lrt.HIT16_DTYPE)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    finally:
        s.close()
