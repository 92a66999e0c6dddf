"""GPU: the learned proposal.

The tensor-core training step's loss and gradient equal the numpy oracle's
(same BF16 rounding points) to 1e-3 relative; inference equals the oracle's
forward; training lowers the loss; triples collected from plain renders are
well formed; and rendering with the proposal returns the plain kernel's hits
bit for bit (the network only chooses where a brick's walk starts), trained or
not, while the counters show walks that started at the predicted voxel."""
import numpy as np
import pytest

from litert_gb300 import lrt, proposal as pp, scenes
from oracle import mlp_oracle as mo

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def union_scene():
    h, n, v = lrt.sbs_from_sdf(lrt.Sdf(**scenes.union_params()), 5, 8)
    s = lrt.Scene(0)
    g = s.add_sbs(h, n, v)
    s.add_instance(g)
    s.commit_scene()
    s.set_preset(render_mode=lrt.RENDER_MODE_NORMAL, sdf_node_intersect=lrt.INTERSECT_NEWTON)
    yield s
    s.close()


def _synthetic(n, seed=3):
    rng = np.random.default_rng(seed)
    x = rng.uniform(0, 1, (n, 16)).astype(np.float32)
    x[:, 6:14] = rng.normal(0, 0.5, (n, 8))
    t = np.clip(0.3 * x[:, 0] + 0.5 * x[:, 4] - 0.2 * x[:, 8], 0, 1).astype(np.float32)
    return x, t


def test_gradient_matches_oracle(union_scene):
    x, t = _synthetic(4096)
    w = pp.init_weights(7)
    pp.set_weights(union_scene, w)
    pp.set_triples(union_scene, x, t)
    loss, g = pp.gradient(union_scene, 4096)
    lo, go = mo.loss_and_grad(w, x, t)
    assert abs(loss - lo) <= 1e-4 * max(1.0, abs(lo))
    assert np.linalg.norm(g - go) <= 1e-3 * np.linalg.norm(go), np.linalg.norm(g - go) / np.linalg.norm(go)
    for a, b in ((0, 512), (512, 544), (544, 1568), (1568, 1600), (1600, 1633)):
        assert np.linalg.norm(g[a:b] - go[a:b]) <= 2e-3 * np.linalg.norm(go[a:b]) + 1e-7, (a, b)


def test_inference_matches_oracle(union_scene):
    x, t = _synthetic(1000, seed=4)
    w = pp.init_weights(8)
    pp.set_weights(union_scene, w)
    pp.set_triples(union_scene, x, t)
    y = pp.infer(union_scene, 0, 1000)
    _, _, _, yo = mo.forward(w, x)
    assert np.linalg.norm(y - yo) <= 3e-3 * np.linalg.norm(yo)
    assert np.abs(y - yo).max() <= 2e-2 * np.abs(yo).max()


@pytest.mark.parametrize("n", [1, 127, 128, 1000, 70000])
def test_tcgen05_inference_matches(union_scene, n):
    """The 128-sample tcgen05/TMEM tiles give the warp-level mma.sync outputs
    (same BF16 rounding points; FP32 sums in the tensor core may be ordered
    differently) and the oracle's forward, including a ragged last tile."""
    x, t = _synthetic(n, seed=11)
    w = pp.init_weights(9)
    pp.set_weights(union_scene, w)
    pp.set_triples(union_scene, x, t)
    y_mma = pp.infer(union_scene, 0, n, engine=pp.ENGINE_MMA)
    y_tc = pp.infer(union_scene, 0, n, engine=pp.ENGINE_TCGEN05)
    _, _, _, yo = mo.forward(w, x)
    scale = max(np.abs(yo).max(), 1e-6)
    assert np.abs(y_tc - y_mma).max() <= 1e-2 * scale, np.abs(y_tc - y_mma).max() / scale
    assert np.linalg.norm(y_tc - yo) <= 3e-3 * np.linalg.norm(yo) + 1e-6
    # an offset window reads the right rows
    if n > 256:
        y_off = pp.infer(union_scene, 100, n - 200, engine=pp.ENGINE_TCGEN05)
        assert np.abs(y_off - y_tc[100:n - 100]).max() <= 1e-2 * scale


def test_tcgen05_inference_trained(union_scene):
    """After training (weights of varied sign and size), the two engines still agree."""
    x, t = _synthetic(20000, seed=12)
    pp.set_weights(union_scene, pp.init_weights(7))
    pp.set_triples(union_scene, x, t)
    pp.train(union_scene, 200, batch=1024, lr=1e-3, seed=3)
    w = pp.get_weights(union_scene)
    y_mma = pp.infer(union_scene, 0, 20000, engine=pp.ENGINE_MMA)
    y_tc = pp.infer(union_scene, 0, 20000, engine=pp.ENGINE_TCGEN05)
    _, _, _, yo = mo.forward(w, x)
    scale = np.abs(yo).max()
    assert np.abs(y_tc - y_mma).max() <= 1e-2 * scale
    assert np.linalg.norm(y_tc - yo) <= 3e-3 * np.linalg.norm(yo)


def test_training_lowers_loss(union_scene):
    x, t = _synthetic(20000, seed=5)
    pp.set_weights(union_scene, pp.init_weights(7))
    pp.set_triples(union_scene, x, t)
    losses = pp.train(union_scene, 400, batch=1024, lr=1e-3, seed=7)
    assert np.isfinite(losses).all()
    assert losses[-20:].mean() < 0.2 * losses[:20].mean(), (losses[:5], losses[-5:])


def test_collect_triples(union_scene):
    views = scenes.union_views(n_views=2, lo=128, hi=192, cam_seed=6)
    pp.set_weights(union_scene, pp.init_weights(7))
    pp.clear(union_scene)
    n = pp.collect(union_scene, views, capacity=200000)
    hits = union_scene.render_host(views, hits=True)["hits"]
    assert n == int((hits["primId"] != lrt.MISS).sum())
    f, t = pp.get_triples(union_scene, 0, n)
    assert np.all((t >= -1e-6) & (t <= 1 + 1e-6))
    assert np.all((f[:, :6] >= -1e-2) & (f[:, :6] <= 1 + 1e-2))
    assert np.all(f[:, 14] > 0)


@pytest.mark.parametrize("trained", [False, True])
def test_proposal_render_equals_plain(union_scene, trained):
    views = scenes.union_views(n_views=4, lo=160, hi=320, cam_seed=8)
    plain = union_scene.render_host(views, hits=True)["hits"].view(np.uint32).copy()
    pp.set_weights(union_scene, pp.init_weights(7))
    if trained:
        pp.clear(union_scene)
        n = pp.collect(union_scene, scenes.union_views(n_views=6, lo=160, hi=320, cam_seed=6), capacity=1_000_000)
        assert n > 10000
        pp.train(union_scene, 600, batch=4096, lr=1e-3, seed=7)
    pp.stats(union_scene)
    union_scene.set_tuning("proposal", 1)
    try:
        got = union_scene.render_host(views, hits=True)["hits"].view(np.uint32).copy()
        st = pp.stats(union_scene)
    finally:
        union_scene.set_tuning("proposal", 0)
    assert np.array_equal(got, plain)
    assert st["proposals"] > 1000
    if trained:
        assert st["jumps"] > 0.05 * st["proposals"], st


def test_trained_network_skips_voxel_steps(union_scene):
    """What training gains: the voxel steps the certified jumps skip, with the
    initial network against the trained one (about 1.5x more after 600 steps on
    these views), while the records stay identical to the plain kernel's."""
    views = scenes.union_views(n_views=4, lo=160, hi=320, cam_seed=8)
    plain = union_scene.render_host(views, hits=True)["hits"].view(np.uint32).copy()
    res = {}
    for trained in (False, True):
        pp.set_weights(union_scene, pp.init_weights(7))
        if trained:
            pp.clear(union_scene)
            pp.collect(union_scene, scenes.union_views(n_views=6, lo=160, hi=320, cam_seed=6), capacity=1_000_000)
            pp.train(union_scene, 600, batch=4096, lr=1e-3, seed=7)
        pp.stats(union_scene)
        union_scene.set_tuning("proposal", 1)
        try:
            got = union_scene.render_host(views, hits=True)["hits"].view(np.uint32).copy()
            res[trained] = pp.stats(union_scene)
        finally:
            union_scene.set_tuning("proposal", 0)
        assert np.array_equal(got, plain)
    assert res[True]["steps_skipped"] > 1.2 * res[False]["steps_skipped"] + 1000, res
    assert res[True]["steps_skipped"] >= res[True]["jumps"]


def test_tcgen05_matches_mma_on_collected_triples(union_scene):
    """Both tensor-core engines issue the same sums (products, then the bias's
    three BF16 terms against a block of ones, all accumulated in FP32 in the
    tensor core; ReLU, BF16): on triples collected from plain renders and a
    trained network their outputs agree to 1e-3 of the output range."""
    pp.set_weights(union_scene, pp.init_weights(7))
    pp.clear(union_scene)
    n = pp.collect(union_scene, scenes.union_views(n_views=6, lo=192, hi=320, cam_seed=6), capacity=2_000_000)
    assert n > 50000
    pp.train(union_scene, 600, batch=4096, lr=1e-3, seed=7)
    y_mma = pp.infer(union_scene, 0, n, engine=pp.ENGINE_MMA)
    y_tc = pp.infer(union_scene, 0, n, engine=pp.ENGINE_TCGEN05)
    rng = float(y_mma.max() - y_mma.min())
    d = np.abs(y_tc - y_mma)
    print(f"{n} triples: max |tcgen05 - mma.sync| = {d.max():.3e} ({d.max() / rng:.3e} of the range), "
          f"{int((d > 0).sum())} outputs differ")
    assert d.max() <= 1e-3 * rng


def test_first_finder_voxel_target(union_scene):
    """The "proposal_target" tuning key 1: the same (ray, brick) triples and
    features, each labelled with the middle of the first voxel the walk runs the
    finder in (as a fraction of the segment) instead of the crossing; a network
    trained on it renders the plain kernel's records bit for bit."""
    views = scenes.union_views(n_views=2, lo=128, hi=192, cam_seed=6)
    pp.set_weights(union_scene, pp.init_weights(7))
    pp.clear(union_scene)
    n0 = pp.collect(union_scene, views, capacity=200000)
    f0, t0 = pp.get_triples(union_scene, 0, n0)
    union_scene.set_tuning("proposal_target", 1)
    try:
        pp.clear(union_scene)
        n1 = pp.collect(union_scene, views, capacity=200000)
    finally:
        union_scene.set_tuning("proposal_target", 0)
    f1, t1 = pp.get_triples(union_scene, 0, n1)
    assert n1 == n0 and n0 > 1000
    order0, order1 = np.lexsort(f0.T), np.lexsort(f1.T)   # collection order is not fixed
    assert np.array_equal(f0[order0], f1[order1])
    assert np.all((t1 >= 0.0) & (t1 <= 1.0 + 1e-6))
    assert not np.array_equal(np.sort(t0), np.sort(t1))
    pp.train(union_scene, 400, batch=4096, lr=1e-3, seed=7)
    test_views = scenes.union_views(n_views=2, lo=160, hi=256, cam_seed=8)
    plain = union_scene.render_host(test_views, hits=True)["hits"].view(np.uint32).copy()
    union_scene.set_tuning("proposal", 1)
    try:
        got = union_scene.render_host(test_views, hits=True)["hits"].view(np.uint32).copy()
    finally:
        union_scene.set_tuning("proposal", 0)
    assert np.array_equal(got, plain)
