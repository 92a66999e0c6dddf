"""CPU: the oracle's Regularization and Redistance (diff_render/MultiRendererDR.cpp
:1933-2055, :2058-2330; the reference cannot be compiled there, so these are
checked against their definitions): the regularisation gradient against a numpy
restatement of the same loops, and redistancing of a distance field scaled by 3
back to |grad| = 1 (within a voxel of the true sphere distance) with the nodes at
the surface untouched."""
import numpy as np
import pytest

from litert_gb300 import dr, lrt, scenes
from oracle import oracle as orc
from oracle import oracle_dr as od


def _grid():
    up = scenes.union_params()
    hdr, nodes, values, params = dr.grid_sbs(3, 2, lrt.Sdf(up["spheres"], up["boxes"], up["k"]), None)
    return hdr, nodes, values, params


@pytest.mark.parametrize("power", [2.0, 3.0])
def test_regularization_matches_restatement(power):
    hdr, nodes, values, params = _grid()
    sc = od.DrScene(orc.SbsHeader(hdr.brick_size, hdr.brick_pad, hdr.bytes_per_value, hdr.aux_data), nodes, values,
                    params.size)
    pr = od.make_preset(reg_function=1, reg_lambda=0.25, reg_power=power)
    got = sc.regularize(params, pr)
    want = np.zeros(params.size, np.float32)
    v = hdr.brick_size + 1
    lam, pw = np.float32(0.25), np.float32(power)
    for node in nodes:
        off = int(node[2])
        for i0 in range(v):
            for j0 in range(v):
                for k0 in range(v):
                    idx = off + i0 * v * v + j0 * v + k0
                    nbs = []
                    if i0 > 0: nbs.append(idx - v * v)
                    if i0 < v - 1: nbs.append(idx + v * v)
                    if j0 > 0: nbs.append(idx - v)
                    if j0 < v - 1: nbs.append(idx + v)
                    if k0 > 0: nbs.append(idx - 1)
                    if k0 < v - 1: nbs.append(idx + 1)
                    for nb in nbs:
                        d = np.float32(params[values[idx]] - params[values[nb]])
                        sgn = np.float32(1.0) if d > 0 else np.float32(-1.0)
                        d = np.float32(abs(d))
                        c = np.float32(np.float32(np.float32(lam * pw) * sgn) * np.float32(np.power(d, pw - np.float32(1))))
                        want[values[idx]] = np.float32(want[values[idx]] + c)
    assert np.abs(got).max() > 0
    assert np.array_equal(got, want)


def test_redistance_restores_unit_gradient():
    n = 33
    h = 2.0 / n
    ax = np.linspace(-1, 1, n, dtype=np.float32)
    X, Y, Z = np.meshgrid(ax, ax, ax, indexing="ij")
    true = np.sqrt(X ** 2 + Y ** 2 + Z ** 2) - 0.5
    scaled = (3.0 * true).astype(np.float32).reshape(-1)
    out = od.redistance(scaled, n, h, n).reshape(n, n, n)
    sc = scaled.reshape(n, n, n)
    # nodes next to a sign change keep their (scaled) values
    near = np.zeros_like(sc, bool)
    for ax_ in range(3):
        a = np.roll(sc, 1, ax_) * sc < 0
        b = np.roll(sc, -1, ax_) * sc < 0
        near |= a | b
    inner = np.zeros_like(near)
    inner[1:-1, 1:-1, 1:-1] = True
    assert np.array_equal(out[near & inner], sc[near & inner])
    far = inner & ~near
    err = np.abs(out[far] - true[far])
    # within about a voxel (the reference's spacing 2/n is a little below the grid's 2/(n-1),
    # and the frozen nodes next to the surface keep their scaled values)
    assert np.median(err) < h and err.max() < 2 * h, (np.median(err) / h, err.max() / h)
    assert np.abs(sc[far] - true[far]).max() > 10 * h   # it was far off before
