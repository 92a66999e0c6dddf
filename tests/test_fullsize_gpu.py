"""GPU parity at the benchmark's full sizes, on samples the oracle finishes in
seconds.

* Headline scene: the 1024^3 smooth union (213,585 bricks of 8^3) rendered in all
  16 uneven views (33.6 M rays) in one batched launch.  The bit-exact kernel's
  records equal the oracle's on every one of the 33.6 M pixels (the oracle on all
  host cores, about 2 s on 16): the same hit mask, t and normal bit for bit, and
  the same brick apart from crossings exactly on a shared brick face, where t is
  equal (measured: 21 of 33.6 M); the contracted kernel meets the forward
  tolerance against the bit-exact one on all rays (hit mask and depth within 1e-4
  of the scene extent apart from < 0.01 % grazing rays).
* Reconstruction: the 8-view 512^2 workload on the 128^3 grid (2.25 M
  parameters); one view's gradient (interior + border integral) equals the
  oracle's within 1e-3 of its norm.
"""
import os

import numpy as np
import pytest

from litert_gb300 import dr, lrt, scenes
from oracle import oracle as orc
from oracle import oracle_dr as od

from _util import canon_bits

pytestmark = pytest.mark.gpu


def test_headline_scene_full_size():
    h, nodes, values = lrt.sbs_from_sdf(scenes.union_sdf(), 7, 8, gpu=0)
    assert nodes.shape[0] > 200000
    s = lrt.Scene(0)
    g = s.add_sbs(h, nodes, values)
    s.add_instance(g)
    s.commit_scene()
    s.set_preset(render_mode=lrt.RENDER_MODE_NORMAL, sdf_node_intersect=lrt.INTERSECT_NEWTON)
    views = scenes.union_views()
    n_rays = sum(w * hh for w, hh, _, _ in views)
    assert n_rays > 30_000_000
    s.set_tuning("fma", 0)
    exact = s.render_host(views, hits=True)["hits"]
    s.set_tuning("fma", 1)
    fused = s.render_host(views, hits=True)["hits"]
    s.close()
    # the bit-exact kernel against the oracle on every pixel
    osc = orc.Scene("sbs", sbs=(orc.SbsHeader(h.brick_size, h.brick_pad, h.bytes_per_value, h.aux_data), nodes,
                                values), intersect=lrt.INTERSECT_NEWTON, render_mode=lrt.RENDER_MODE_NORMAL)
    n_cmp = n_hit = n_face = 0
    off = 0
    for w, hh, wv, pj in views:
        pix = np.arange(w * hh, dtype=np.uint32)
        o, _ = osc.render_pixels(w, hh, lrt.inverse4x4(pj), lrt.inverse4x4(wv), pix, threads=os.cpu_count() or 1)
        gsel = exact[off:off + w * hh]
        off += w * hh
        mo = o["primId"] != lrt.MISS
        assert np.array_equal(gsel["primId"] != lrt.MISS, mo)
        assert np.array_equal(canon_bits(gsel["t"][mo]), canon_bits(o["t"][mo]))
        # bricks do not overlap: equal t in two bricks needs a crossing exactly on a shared face
        same = mo & (gsel["primId"] == o["primId"])
        n_face += int((mo & ~same).sum())
        assert np.array_equal(canon_bits(gsel["nx"][same]), canon_bits(o["coords"][same, 2]))
        assert np.array_equal(canon_bits(gsel["ny"][same]), canon_bits(o["coords"][same, 3]))
        n_cmp += pix.size
        n_hit += int(mo.sum())
    assert n_cmp == n_rays and n_hit > 5_000_000
    assert n_face <= 1e-6 * n_rays, n_face
    # the contracted kernel against the bit-exact one on every ray: rays whose hit or
    # depth differs (beyond 1e-4 of the extent 2) are grazing rays -- a tangent
    # crossing found by one kernel and missed by the other, the ray going on to a
    # surface behind -- and stay within the 0.01 % grazing allowance (measured: 1
    # mask and 7 depth differences in 33.6 M rays)
    me, mf = exact["primId"] != lrt.MISS, fused["primId"] != lrt.MISS
    assert me.sum() > 5_000_000
    both = me & mf
    far = np.abs(exact["t"][both].astype(np.float64) - fused["t"][both]) > 1e-4 * 2.0
    assert int((me != mf).sum()) + int(far.sum()) <= 1e-4 * n_rays
    assert far.sum() <= 1e-6 * n_rays


def test_reconstruction_gradient_full_size():
    target, init, views = scenes.dr_workload()
    R = dr.MultiRendererDR()
    R.SetScene(*target)
    R.SetPreset(dr.default_preset(reconstruction_flags=0, border_spp=0))
    R.SetReference([np.zeros((v[1], v[0], 4), np.float32) for v in views], [v[2] for v in views],
                   [v[3] for v in views])
    imgs = []
    for i in range(len(views)):
        R.render_grad(i)
        imgs.append(R.getLastImage(i).copy())
    R.SetScene(*init)
    R.SetReference(imgs, [v[2] for v in views], [v[3] for v in views])
    preset = dr.default_preset(opt_lr=3e-3, spp=1, border_spp=256, seed=1)
    R.SetPreset(preset)
    assert init[3].size > 2_000_000
    _, g = R.render_grad(3)
    hdr, nodes, values, params = init
    osc = od.DrScene(orc.SbsHeader(hdr.brick_size, hdr.brick_pad, hdr.bytes_per_value, hdr.aux_data), nodes, values,
                     params.size, pairs=R.bvh2())
    lights = [(preset.lights[i].type, np.array(preset.lights[i].dir[:], np.float32),
               np.array(preset.lights[i].color[:], np.float32)) for i in range(preset.n_lights)]
    op = od.make_preset(render_mode=preset.render_mode, reconstruction=preset.reconstruction_flags, spp=1,
                        border_spp=256, seed=1, lights=lights, lr=preset.opt_lr)
    w, hh, wv, pj = views[3]
    o = osc.render(params, op, od.make_view(w, hh, wv, pj, lrt.inverse4x4), imgs[3].reshape(-1, 4))
    R.close()
    nrm = np.linalg.norm(o["grad"])
    assert nrm > 0
    assert np.linalg.norm(g - o["grad"]) <= 1e-3 * nrm
