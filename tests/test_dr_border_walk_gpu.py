"""GPU: the border integral's voxel walk against the reference's.

The border kernel's walk skips, from the first voxel on, every voxel and brick
whose corner values all exceed min(relaxation SDF, border_relax_eps) plus a
rounding margin, and walks a ray again in full wherever that could change its
record (only rays whose relaxation SDF ends below border_relax_eps contribute to
the border integral).  lrt_dr_query_rays with flag bit 32 runs that walk; here
its records are held to the oracle's RayQuery_NearestHitWithGrad border walk
(diff_render/BVH2DR.cpp:12-102, 623-1073), which skips nothing:

* the hit (t, primId, colour, normal) of every ray, bit for bit;
* which rays end below border_relax_eps, exactly;
* for those rays, the whole relaxation record (t, sdf, colour, normal, the 8
  parameter indices and dSDF/dtheta), bit for bit.

Two scenes: the dense grid (bricks share their face values, so the field is
continuous across bricks) and the same grid with every brick's distances made
private and perturbed independently, so the field jumps across brick faces --
the case where a voxel-entry update (check_vox_border) at a brick's first voxel
can differ between the walks and the re-walk has to catch it."""
import numpy as np
import pytest

from litert_gb300 import dr, lrt, scenes
from oracle import oracle as orc
from oracle import oracle_dr as od

pytestmark = pytest.mark.gpu


def _scene(private, seed=11):
    up = scenes.union_params()
    hdr, nodes, values, params = dr.grid_sbs(6, 4, lrt.Sdf(up["spheres"], up["boxes"], up["k"]), None)
    rng = np.random.default_rng(seed)
    params = params.copy()
    if not private:
        nd = 25 ** 3
        params[:nd] += rng.normal(0, 0.004, nd).astype(np.float32)
        return hdr, nodes, values, params
    v3 = (hdr.brick_size + 2 * hdr.brick_pad + 1) ** 3
    values = values.copy()
    base = params.size
    extra = []
    for b in range(nodes.shape[0]):
        off = int(nodes[b, 2])
        idx = values[off:off + v3].astype(np.int64)
        extra.append(params[idx] + rng.normal(0, 0.01, v3).astype(np.float32))
        values[off:off + v3] = base + b * v3 + np.arange(v3, dtype=np.uint32)
    return hdr, nodes, values, np.concatenate([params, np.concatenate(extra).astype(np.float32)])


def _rays(rng, n_random=6000):
    pj = lrt.perspective(45.0, 1.0, 0.01, 100.0)
    P, D = [], []
    for i in range(3):
        a = 2 * np.pi * i / 3 + 0.3
        wv = lrt.look_at([2.6 * np.sin(a), 1.0, 2.6 * np.cos(a)], [0, 0, 0], [0, 1, 0])
        p_, d_ = orc.eye_rays(96, 96, lrt.inverse4x4(pj), lrt.inverse4x4(wv), np.arange(96 * 96, dtype=np.uint32),
                              0.37, 0.61)
        P.append(p_)
        D.append(d_)
    rp = np.zeros((n_random, 4), np.float32)
    rp[:, :3] = rng.uniform(-1.6, 1.6, (n_random, 3))
    rd = np.zeros((n_random, 4), np.float32)
    d = rng.normal(size=(n_random, 3))
    rd[:, :3] = d / np.linalg.norm(d, axis=1, keepdims=True)
    rd[:, 3] = 1e9
    P.append(rp)
    D.append(rd)
    return np.concatenate(P), np.concatenate(D)


@pytest.mark.parametrize("private", [False, True])
@pytest.mark.parametrize("eps", [1e-3, 2e-2])
def test_border_integral_walk_matches_reference_walk(private, eps):
    hdr, nodes, values, params = _scene(private)
    P, D = _rays(np.random.default_rng(5))
    R = dr.MultiRendererDR()
    try:
        R.SetScene(hdr, nodes, values, params)
        R.SetPreset(dr.default_preset(render_mode=dr.RENDER_LAMBERT, border_relax_eps=eps))
        flags = 1 | 8   # colour derivatives on the hit, the border relaxation point
        got = R.query_rays(flags | 32, P, D)
        full = R.query_rays(flags, P, D)
        osc = od.DrScene(orc.SbsHeader(hdr.brick_size, hdr.brick_pad, hdr.bytes_per_value, hdr.aux_data), nodes,
                         values, params.size, pairs=R.bvh2(), need_normal=True)
        o = osc.query(params, flags, P, D).view(np.uint32).reshape(len(P), -1)
    finally:
        R.close()
    want = np.concatenate([o[:, [0, 1]], o[:, 4:7], o[:, 8:11], o[:, [14, 21]], o[:, 18:21], o[:, 22:25],
                           o[:, 28:36], o[:, 36:44]], 1)
    # the engine's full walk is the oracle's, record for record
    assert np.array_equal(full, want)
    assert (want[:, 1] != 0xFFFFFFFF).sum() > 3000
    # the hit of every ray
    assert np.array_equal(got[:, :8], want[:, :8])
    # which rays end below relax_eps, and their whole relaxation records
    below = want[:, 9].view(np.float32) < np.float32(eps)
    assert below.sum() > 50
    assert np.array_equal(got[:, 9].view(np.float32) < np.float32(eps), below)
    bad = np.nonzero((got[below] != want[below]).any(1))[0]
    assert bad.size == 0, (bad.size, got[below][bad[:2]], want[below][bad[:2]])
