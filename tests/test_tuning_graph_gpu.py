"""GPU: launch-shape tuning, the autotuner and CUDA-graph replay of the batched
render.  Every tile shape / stack depth / kernel variant gives the same hit
records bit for bit; a replayed graph equals a direct render, also after its
cameras change; the autotuner picks one of its candidates and leaves results
unchanged."""
import numpy as np
import pytest
import torch

from litert_gb300 import lrt, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scene():
    h, n, v = lrt.sbs_from_sdf(lrt.Sdf(**scenes.union_params()), 5, 8)
    s = lrt.Scene(0)
    g = s.add_sbs(h, n, v)
    s.add_instance(g)
    s.commit_scene()
    s.set_preset(render_mode=lrt.RENDER_MODE_NORMAL, sdf_node_intersect=lrt.INTERSECT_NEWTON)
    yield s
    s.close()


def _views():
    return scenes.union_views(n_views=5, lo=96, hi=300)


def _render(s, views):
    return s.render_host(views, hits=True)["hits"].view(np.uint32).copy()


@pytest.mark.parametrize("tile_w,stack,variant", [(4, 64, 0), (16, 64, 0), (32, 64, 0), (8, 32, 0), (8, 64, 1),
                                                  (16, 32, 0), (8, 64, 2), (4, 32, 2), (16, 64, 2), (8, 64, 3),
                                                  (4, 64, 3), (8, 32, 3), (32, 64, 3)])
def test_launch_shapes_bit_identical(scene, tile_w, stack, variant):
    views = _views()
    ref = _render(scene, views)
    scene.set_tuning("tile_w", tile_w)
    scene.set_tuning("stack", stack)
    scene.set_tuning("variant", variant)
    try:
        got = _render(scene, views)
    finally:
        scene.set_tuning("tile_w", 8)
        scene.set_tuning("stack", 64)
        scene.set_tuning("variant", 0)
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("refill", [1, 4, 16, 32])
def test_refill_variant_bit_identical(scene, refill):
    views = _views()
    ref = _render(scene, views)
    scene.set_tuning("variant", 2)
    scene.set_tuning("refill", refill)
    try:
        got = _render(scene, views)
    finally:
        scene.set_tuning("variant", 0)
        scene.set_tuning("refill", 8)
    assert np.array_equal(got, ref)


def test_refill_variant_triangles():
    verts, faces = scenes.displaced_icosphere(subdiv=4)
    s = lrt.Scene(0)
    g = s.add_triangles(verts, faces)
    s.add_instance(g)
    s.commit_scene()
    s.set_preset(render_mode=lrt.RENDER_MODE_NORMAL)
    view = [scenes.mesh_view(width=320, height=200)]
    a = s.render_host(view, hits=True, rgba=True)
    s.set_tuning("variant", 2)
    b = s.render_host(view, hits=True, rgba=True)
    s.close()
    assert np.array_equal(a["hits"].view(np.uint32), b["hits"].view(np.uint32))
    assert np.array_equal(a["rgba"].view(np.uint32), b["rgba"].view(np.uint32))


def test_graph_replay_matches_render(scene):
    views = _views()
    n = sum(w * h for w, h, _, _ in views)
    ref = _render(scene, views)
    out = torch.zeros(n * 4, dtype=torch.float32, device="cuda")
    g = scene.graph_create(views, hits_ptr=out.data_ptr())
    try:
        for _ in range(3):
            out.zero_()
            scene.graph_launch(g)
            torch.cuda.synchronize()
            assert np.array_equal(out.cpu().numpy().view(np.uint32), ref)
        moved = scenes.union_views(n_views=5, lo=96, hi=300, cam_seed=11)
        moved = [(w, h, mv[2], mv[3]) for (w, h, _, _), mv in zip(views, moved)]
        scene.graph_set_views(g, moved)
        scene.graph_launch(g)
        torch.cuda.synchronize()
        assert np.array_equal(out.cpu().numpy().view(np.uint32), _render(scene, moved))
        with pytest.raises(lrt.LrtError):
            scene.graph_set_views(g, moved[:4])
    finally:
        lrt.Scene.graph_destroy(g)


def test_autotune_picks_a_candidate(scene):
    views = _views()
    ref = _render(scene, views)
    best, tried = scene.autotune(views, reps=2)
    assert len(tried) >= 6
    assert best["ms"] == min(c["ms"] for c in tried)
    assert best["tile_w"] in (4, 8, 16) and best["stack"] in (32, 64)
    assert np.array_equal(_render(scene, views), ref)


@pytest.mark.parametrize("fma", [0, 1])
def test_render_into_page_locked_host_memory(scene, fma):
    """lrt_render_host writes page-locked outputs from the kernel directly; the
    records, colours and packed colours equal those of the copy path
    (pageable numpy buffers)."""
    scene.set_tuning("fma", fma)
    try:
        views = _views()
        n = sum(w * h for w, h, _, _ in views)
        ref = scene.render_host(views, hits=True, rgba=True, rgba8=True)
        hits = torch.full((n * 4,), -1.0, dtype=torch.float32, pin_memory=True)
        rgba = torch.full((n * 4,), -1.0, dtype=torch.float32, pin_memory=True)
        rgba8 = torch.zeros((n,), dtype=torch.int32, pin_memory=True)
        va = lrt.make_views(views)
        st = lrt.lib().lrt_render_host(scene._ctx, lrt.C.cast(va, lrt.C.c_void_p), len(views),
                                       lrt.C.c_void_p(hits.data_ptr()), lrt.C.c_void_p(rgba.data_ptr()),
                                       lrt.C.c_void_p(rgba8.data_ptr()))
        assert st == 0
        assert np.array_equal(hits.numpy().view(np.uint32), ref["hits"].view(np.uint32))
        assert np.array_equal(rgba.numpy().view(np.uint32), ref["rgba"].view(np.uint32).reshape(-1))
        assert np.array_equal(rgba8.numpy().view(np.uint32), ref["rgba8"])
    finally:
        scene.set_tuning("fma", 0)


@pytest.mark.parametrize("mode", [lrt.RENDER_MODE_LAMBERT_NO_TEX, lrt.RENDER_MODE_DEPTH])
def test_regrouped_variant_colours_and_rgba8(scene, mode):
    """Variant 3 (traversal and leaf phases regrouped across the block) gives the
    per-lane kernel's records, float colours and packed RGBA8 bit for bit."""
    views = _views()
    scene.set_preset(render_mode=mode)
    try:
        ref = scene.render_host(views, hits=True, rgba=True, rgba8=True)
        scene.set_tuning("variant", 3)
        got = scene.render_host(views, hits=True, rgba=True, rgba8=True)
    finally:
        scene.set_tuning("variant", 0)
        scene.set_preset(render_mode=lrt.RENDER_MODE_NORMAL)
    for k in ("hits", "rgba", "rgba8"):
        assert np.array_equal(np.ascontiguousarray(got[k]).view(np.uint32), np.ascontiguousarray(ref[k]).view(np.uint32)), k
