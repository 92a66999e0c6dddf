"""CPU: OptimizeGrid's grids (diff_render/MultiRendererDR.cpp:228-276).  The
engine's create_grid_sbs with the grid sampler and gradient colours equals the
oracle's restatement bit for bit (starting grid and resampled grids, growing or
not), reproduces a linear distance field inside the cube (trilinear
interpolation is exact for it; on the +1 faces the sampler takes the lower grid
corner's value), and lays out nodes and indices as the SDF-sampled grid of the same shape."""
import numpy as np
import pytest

from litert_gb300 import dr, lrt
from oracle import oracle_dr as od


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


@pytest.mark.parametrize("gs", [2, 4, 5])
def test_starting_grid_matches_oracle(gs):
    _, _, _, p = dr.grid_resample(gs, 1)
    assert np.array_equal(_bits(p), _bits(od.grid_resample(gs, 1)))


@pytest.mark.parametrize("gs,old_bs,bs", [(4, 1, 2), (4, 2, 4), (3, 2, 2), (2, 4, 8)])
def test_resampled_grid_matches_oracle(gs, old_bs, bs):
    rng = np.random.default_rng(gs * 100 + bs)
    n_old = (gs * old_bs + 1) ** 3 + 3 * (gs + 1) ** 3
    old = rng.normal(0, 0.3, n_old).astype(np.float32)
    _, _, _, p = dr.grid_resample(gs, bs, old, old_bs)
    assert np.array_equal(_bits(p), _bits(od.grid_resample(gs, bs, old, old_bs)))


def test_resample_reproduces_a_linear_field():
    gs, old_bs, bs = 4, 2, 4
    a, b = np.array([0.3, -0.2, 0.5], np.float32), np.float32(0.1)

    def coords(s):
        t = 2.0 * (np.arange(gs * s + 1, dtype=np.float32) / np.float32(gs * s)) - 1.0
        return np.stack(np.meshgrid(t, t, t, indexing="ij"), -1).reshape(-1, 3)

    n_old = (gs * old_bs + 1) ** 3
    old = np.zeros(n_old + 3 * (gs + 1) ** 3, np.float32)
    old[:n_old] = coords(old_bs) @ a + b
    _, _, _, p = dr.grid_resample(gs, bs, old, old_bs)
    q = coords(bs)
    want = q @ a + b
    # points on a +1 face take the grid_sampler's other branch: the value at the
    # lower grid corner, without interpolation (:258-261)
    inner = np.all(q < 1.0, axis=1)
    assert inner.sum() == (gs * bs) ** 3
    assert np.max(np.abs(p[:want.size][inner] - want[inner])) < 1e-5
    edge = ~inner
    lo = np.floor((0.5 * (q[edge] + 1.0)) * gs * old_bs + 1e-6).astype(int)
    lo = np.minimum(lo, gs * old_bs)
    t = 2.0 * (lo.astype(np.float32) / np.float32(gs * old_bs)) - 1.0
    assert np.max(np.abs(p[:want.size][edge] - (t @ a + b))) < 1e-5


def test_layout_matches_sdf_grid():
    h1, n1, v1, _ = dr.grid_resample(3, 2)
    h2, n2, v2, _ = dr.grid_sbs(3, 2, lrt.Sdf(spheres=np.array([[0, 0, 0, 0.5]], np.float32)), None)
    assert (h1.brick_size, h1.aux_data) == (h2.brick_size, h2.aux_data)
    assert np.array_equal(n1, n2) and np.array_equal(v1, v2)
