"""CPU: the oracle's SVM border sampling helpers (CastBorderRaySVM,
diff_render/MultiRendererDR.cpp:1518-1931).  The reference's MultiRendererDR.cpp
cannot be compiled here (it needs the image library and the renderer), so the
helpers are checked against their definitions: SVM_fit against a numpy float32
restatement of the same loop (bit for bit), CohenSutherlandLineClip on segments
whose clipped ends are known, and the per-pixel sampling line on a rendered
sphere: interior pixels get no line, silhouette pixels get a stripe through the
pixel."""
import numpy as np
import pytest

from litert_gb300 import dr, lrt
from oracle import oracle as orc
from oracle import oracle_dr as od


def _svm_fit_np(rows):
    """SVM_fit restated with numpy float32 scalars (etha 0.01, alpha 0.1, 200 epochs)."""
    f = np.float32
    X = np.asarray(rows, np.float32) * f(0.01)
    etha, alpha = f(0.01), f(0.1)
    mult = f(1.0) - etha * alpha / f(200)
    w = [f(-1.0), f(1.0), f(0.0)]
    errors = X.shape[0]
    e = 0
    while e < 200 and errors > 0:
        errors = 0
        for j in range(X.shape[0]):
            margin = w[0] * X[j, 0] + w[1] * X[j, 1] + w[2] * X[j, 2]
            w = [w[0] * mult, w[1] * mult, w[2] * mult]
            if margin < 0:
                w = [w[0] + X[j, 0], w[1] + X[j, 1], w[2] + X[j, 2]]
                errors += 1
        e += 1
    return np.array([w[0], w[1], w[2], f(errors) / f(X.shape[0])], np.float32)


def _rows(pts, labels):
    return (np.c_[pts, np.ones(len(pts))] * labels[:, None]).astype(np.float32)


@pytest.mark.parametrize("seed,separable", [(0, True), (1, True), (2, False)])
def test_svm_fit_matches_restatement(seed, separable):
    rng = np.random.default_rng(seed)
    pts = rng.uniform(0, 1, (64, 2)).astype(np.float32)
    a = rng.uniform(-1, 1)
    lab = np.where(pts[:, 1] - 0.5 - a * (pts[:, 0] - 0.5) < 0, -1.0, 1.0).astype(np.float32)
    if not separable:
        lab[rng.choice(64, 8, replace=False)] *= -1
    W = od.svm_fit(_rows(pts, lab))
    assert np.array_equal(W.view(np.uint32), _svm_fit_np(_rows(pts, lab)).view(np.uint32))
    if separable:
        assert W[3] == 0.0
        m = lab * (W[0] * pts[:, 0] + W[1] * pts[:, 1] + W[2])
        assert np.all(m >= 0)
    else:
        assert W[3] > 0.0


@pytest.mark.parametrize("seg,want", [
    ((-0.5, 0.5, 1.5, 0.5), (True, 0.0, 0.5, 1.0, 0.5)),
    ((0.25, -1.0, 0.25, 2.0), (True, 0.25, 0.0, 0.25, 1.0)),
    ((0.2, 0.3, 0.7, 0.6), (True, 0.2, 0.3, 0.7, 0.6)),
    ((2.0, 2.0, 3.0, 3.0), (False, None, None, None, None)),
    ((-1.0, -1.0, 2.0, 2.0), (True, 0.0, 0.0, 1.0, 1.0)),
    ((-0.5, 1.2, 0.5, 2.0), (False, None, None, None, None)),
])
def test_line_clip(seg, want):
    got = od.line_clip(*seg)
    assert got[0] == want[0]
    if want[0]:
        assert np.allclose(got[1:], want[1:], atol=1e-6)


def test_svm_line_on_a_sphere():
    hdr, nodes, values, params = dr.grid_sbs(4, 4, lrt.Sdf(spheres=np.array([[0, 0, 0, 0.6]], np.float32)),
                                             [0.8, 0.3, 0.2])
    sc = od.DrScene(orc.SbsHeader(hdr.brick_size, hdr.brick_pad, hdr.bytes_per_value, hdr.aux_data), nodes, values,
                    params.size)
    W = H = 32
    pj = lrt.perspective(45.0, 1.0, 0.01, 100.0)
    wv = lrt.look_at([0, 0, 3.0], [0, 0, 0], [0, 1, 0])
    view = od.make_view(W, H, wv, pj, lrt.inverse4x4)
    pr = od.make_preset(border_spp=64, border_sampling=1)
    out = sc.render(params, pr, view, np.zeros((W * H, 4), np.float32), threads=1)
    alpha = out["image"][:, 3].reshape(H, W)
    inside = [(x, y) for y in range(H) for x in range(W) if alpha[y, x] == 1.0 and
              alpha[max(0, y - 1):y + 2, max(0, x - 1):x + 2].min() == 1.0]
    border = out["border"].reshape(H, W)
    edge = [(x, y) for y in range(H) for x in range(W) if border[y, x]]
    assert len(inside) > 20 and len(edge) > 8
    for x, y in inside[:10]:
        assert sc.svm_line(params, pr, view, x, y).count == 0
    # border pixels span the 3x3 neighbourhood of the silhouette; only those the
    # silhouette crosses have classification samples of both kinds and keep a line
    lines = [(x, y, sc.svm_line(params, pr, view, x, y)) for x, y in edge]
    kept = [(x, y, L) for x, y, L in lines if L.count > 0]
    assert len(kept) >= 0.2 * len(edge)
    for x, y, L in kept:
        nb = alpha[max(0, y - 1):y + 2, max(0, x - 1):x + 2]
        assert nb.min() == 0.0 and nb.max() == 1.0
        assert L.svm_spp == 16 and 1 <= L.count <= 64 - 16 and L.pdf > 0
        if not L.force:
            # the stripe's centre line passes through the pixel square
            t = np.linspace(0, 1, 101)
            px, py = L.p0[0] + t * L.r[0], L.p0[1] + t * L.r[1]
            assert np.any((px >= 0) & (px <= 1) & (py >= 0) & (py <= 1))
