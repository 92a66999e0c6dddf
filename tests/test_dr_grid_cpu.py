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


def _preprocess_np(img, width, height):
    """PreprocessRefImages restated with numpy float32 scalars (bilinear, texel centres,
    clamped edges; alpha from the 'colour differs from black' mask)."""
    f = np.float32
    h0, w0 = img.shape[:2]
    rgb = img[..., :3].astype(np.float32)
    m = (np.sqrt(rgb[..., 0] * rgb[..., 0] + rgb[..., 1] * rgb[..., 1] + rgb[..., 2] * rgb[..., 2]) <
         f(0.001)).astype(np.float32)
    mask = np.repeat((f(1) - m)[..., None], 4, axis=2).astype(np.float32)
    sx, sy = int(np.ceil(f(w0) / f(width))), int(np.ceil(f(h0) / f(height)))

    def sample(im, u, v):
        fx, fy = u * f(w0) - f(0.5), v * f(h0) - f(0.5)
        x0f, y0f = np.floor(fx), np.floor(fy)
        tx, ty = fx - x0f, fy - y0f
        xa, xb = min(max(int(x0f), 0), w0 - 1), min(max(int(x0f) + 1, 0), w0 - 1)
        ya, yb = min(max(int(y0f), 0), h0 - 1), min(max(int(y0f) + 1, 0), h0 - 1)
        a, b, d, e = im[ya, xa], im[ya, xb], im[yb, xa], im[yb, xb]
        return (f(1) - ty) * ((f(1) - tx) * a + tx * b) + ty * ((f(1) - tx) * d + tx * e)

    out = np.zeros((height, width, 4), np.float32)
    k = f(sx * sy)
    for y in range(height):
        for x in range(width):
            acc = np.zeros(4, np.float32)
            for dx in range(sx):
                for dy in range(sy):
                    u = (f(sx * x + dx) + f(0.5)) / f(sx * width)
                    v = (f(sy * y + dy) + f(0.5)) / f(sy * height)
                    col = sample(img.astype(np.float32), u, v).astype(np.float32)
                    col[3] = sample(mask, u, v)[3]
                    acc = (acc + col / k).astype(np.float32)
            out[y, x] = acc
    return out


@pytest.mark.parametrize("size", [(7, 5), (16, 16), (30, 11)])
def test_preprocess_reference_matches_restatement(size):
    rng = np.random.default_rng(size[0])
    imgs = [rng.uniform(0, 1, (16, 20, 4)).astype(np.float32) for _ in range(2)]
    imgs[0][3:9, 4:12, :3] = 0.0            # background patches: mask 0 there
    pj = lrt.perspective(45.0, 1.0, 0.01, 100.0)
    views = [(20, 16, lrt.look_at([0, 0, 3], [0, 0, 0], [0, 1, 0]), pj)] * 2
    out_v, out = dr.preprocess_reference(views, imgs, *size)
    assert out_v[0].width == size[0] and out_v[0].height == size[1]
    for k in range(2):
        want = _preprocess_np(imgs[k], *size)
        assert np.array_equal(out[k].view(np.uint32), want.view(np.uint32))
