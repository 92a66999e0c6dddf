"""GPU: lrt_render_host into page-locked host memory.

With "host_copy" 1 (the default) a render whose kernel publishes chunk counts
writes device buffers, and each chunk of whole tile rows is copied to the host
while later tiles render; with "host_copy" 0 the kernel writes the host memory
itself.  Both must give the records and colours of a render into pageable
memory, bit for bit: ragged view sizes, one-pixel views, more views than
chunks of a view, every output at once, the PHONG shading kernel, the
contracted kernel, the first-hit walk, and the packet kernel (which publishes
nothing and keeps the direct writes).  Calls alternate between two view sets
over the same staging buffers, so a chunk copied before its tiles were written
would return the other set's records."""
import numpy as np
import pytest
import torch

from litert_gb300 import lrt, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scene():
    h, n, v = lrt.sbs_from_sdf(lrt.Sdf(**scenes.union_params()), 6, 8)
    s = lrt.Scene(0)
    s.add_instance(s.add_sbs(h, n, v))
    s.commit_scene()
    s.set_preset(render_mode=lrt.RENDER_MODE_NORMAL, sdf_node_intersect=lrt.INTERSECT_NEWTON)
    yield s
    s.close()


def _pinned(shape, dtype):
    nbytes = int(np.prod(shape)) * np.dtype(dtype).itemsize
    t = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    a = t.numpy().view(dtype).reshape(shape)
    a.view(np.uint8)[:] = 0xA5   # not a record the render writes
    return t, a


def _render_pinned(scene, views, hits=True, rgba=False, rgba8=False):
    va = lrt.make_views(views)
    npix = sum(int(w) * int(h) for w, h, _, _ in views)
    keep, out = [], {}
    ptr = []
    for name, on, shape, dt in (("hits", hits, (npix,), lrt.HIT16_DTYPE), ("rgba", rgba, (npix, 4), np.float32),
                                ("rgba8", rgba8, (npix,), np.uint32)):
        if on:
            t, a = _pinned(shape, dt)
            keep.append(t)
            out[name] = a
            ptr.append(lrt.C.c_void_p(a.ctypes.data))
        else:
            ptr.append(None)
    st = lrt.lib().lrt_render_host(scene._ctx, lrt.C.cast(va, lrt.C.c_void_p), len(views), *ptr)
    assert st == 0, lrt.lib().lrt_last_error(scene._ctx)
    return {k: v.copy() for k, v in out.items()}


def _same(a, b):
    for k in a:
        assert np.array_equal(a[k].view(np.uint8), b[k].view(np.uint8)), k


def _check(scene, view_sets, **outs):
    want = [scene.render_host(v, **outs) for v in view_sets]
    for copy in (1, 0):
        scene.set_tuning("host_copy", copy)
        try:
            for rep in range(2):
                for v, w in zip(view_sets, want):
                    _same(_render_pinned(scene, v, **outs), w)
        finally:
            scene.set_tuning("host_copy", 1)


def _views_a():
    return scenes.union_views(n_views=3, size_seed=11, cam_seed=3, lo=200, hi=900)


def _views_b():
    v = scenes.union_views(n_views=3, size_seed=12, cam_seed=4, lo=200, hi=900)
    return v + [(1, 1, v[0][2], v[0][3]), (1000, 3, v[1][2], v[1][3])]


def test_hits_ragged_views(scene):
    _check(scene, [_views_a(), _views_b()])


def test_many_small_views(scene):
    _check(scene, [scenes.union_views(n_views=70, size_seed=13, cam_seed=6, lo=17, hi=140),
                   scenes.union_views(n_views=40, size_seed=14, cam_seed=7, lo=60, hi=300)])


def test_every_output_phong(scene):
    scene.set_preset(render_mode=lrt.RENDER_MODE_PHONG, sdf_node_intersect=lrt.INTERSECT_NEWTON)
    try:
        _check(scene, [_views_a(), _views_b()], hits=True, rgba=True, rgba8=True)
    finally:
        scene.set_preset(render_mode=lrt.RENDER_MODE_NORMAL, sdf_node_intersect=lrt.INTERSECT_NEWTON)


@pytest.mark.parametrize("key,value", [("fma", 1), ("first_hit", 1), ("variant", 1), ("tile_w", 4)])
def test_kernel_choices(scene, key, value):
    scene.set_tuning(key, value)
    try:
        _check(scene, [_views_a(), _views_b()], hits=True, rgba8=True)
    finally:
        scene.set_tuning(key, {"fma": 0, "first_hit": 0, "variant": 0, "tile_w": 8}[key])
