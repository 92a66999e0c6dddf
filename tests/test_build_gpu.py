"""GPU: the SBS and SVS builders on the GPU return the host builders' output
exactly -- the same bricks / voxels, in the same order, with the same quantised
values -- for several depths, brick sizes, paddings and value widths, on the
sphere of the small configuration and on the smooth union of the large one
(including its 1024^3 effective grid: depth 7, 8-voxel bricks)."""
import numpy as np
import pytest

from litert_gb300 import lrt, scenes

pytestmark = pytest.mark.gpu


def _same_sbs(a, b):
    (ha, na, va), (hb, nb, vb) = a, b
    assert (ha.brick_size, ha.brick_pad, ha.bytes_per_value, ha.aux_data) == \
           (hb.brick_size, hb.brick_pad, hb.bytes_per_value, hb.aux_data)
    assert na.shape == nb.shape, (na.shape, nb.shape)
    assert np.array_equal(na, nb)
    assert np.array_equal(va, vb)


@pytest.mark.parametrize("depth,bs,pad,bpv", [(4, 4, 0, 4), (6, 4, 0, 4), (5, 8, 0, 4), (5, 4, 1, 2), (5, 3, 1, 1),
                                              (6, 2, 0, 1), (5, 16, 1, 4)])
def test_sphere_sbs(depth, bs, pad, bpv):
    sdf = lrt.Sdf(**scenes.SPHERE_SDF)
    host = lrt.sbs_from_sdf(sdf, depth, bs, pad, bpv)
    gpu = lrt.sbs_from_sdf(sdf, depth, bs, pad, bpv, gpu=0)
    assert host[1].shape[0] > 10
    _same_sbs(gpu, host)


@pytest.mark.parametrize("depth,bs,pad,bpv", [(5, 8, 0, 4), (6, 4, 1, 1), (7, 8, 0, 4)])
def test_union_sbs(depth, bs, pad, bpv):
    sdf = scenes.union_sdf()
    host = lrt.sbs_from_sdf(sdf, depth, bs, pad, bpv)
    gpu = lrt.sbs_from_sdf(sdf, depth, bs, pad, bpv, gpu=0)
    _same_sbs(gpu, host)


@pytest.mark.parametrize("params,depth", [("sphere", 6), ("sphere", 4), ("union", 7), ("union", 8)])
def test_svs(params, depth):
    sdf = lrt.Sdf(**scenes.SPHERE_SDF) if params == "sphere" else scenes.union_sdf()
    host = lrt.svs_from_sdf(sdf, depth)
    gpu = lrt.svs_from_sdf(sdf, depth, gpu=0)
    assert host.shape[0] > 10
    assert np.array_equal(gpu, host)


def test_shallow_depth_is_refused():
    with pytest.raises(lrt.LrtError):
        lrt.sbs_from_sdf(lrt.Sdf(**scenes.SPHERE_SDF), 3, 4, gpu=0)
    with pytest.raises(lrt.LrtError):
        lrt.svs_from_sdf(lrt.Sdf(**scenes.SPHERE_SDF), 3, gpu=0)


def test_gpu_built_scene_through_a_file_renders_like_the_host_built_one(tmp_path):
    """GPU build -> save (the reference's file layout) -> load -> render equals the
    render of the host-built scene bit for bit."""
    sdf = scenes.union_sdf()
    h, n, v = lrt.sbs_from_sdf(sdf, 5, 8, gpu=0)
    p = tmp_path / "union.sbs"
    lrt.save_sbs(p, h, n, v)
    h2, n2, v2 = lrt.load_sbs(p)
    views = scenes.union_views(n_views=2, lo=128, hi=192, cam_seed=3)
    out = []
    for hh, nn, vv in ((h2, n2, v2), lrt.sbs_from_sdf(sdf, 5, 8)):
        s = lrt.Scene(0)
        s.add_instance(s.add_sbs(hh, nn, vv))
        s.commit_scene()
        s.set_preset(render_mode=lrt.RENDER_MODE_NORMAL, sdf_node_intersect=lrt.INTERSECT_NEWTON)
        out.append(s.render_host(views, hits=True)["hits"].view(np.uint32).copy())
        s.close()
    assert (out[0].reshape(-1, 4)[:, 1] != lrt.MISS).sum() > 1000
    assert np.array_equal(out[0], out[1])
