"""Benchmark: SBS primary-ray throughput (Mrays/s) on the large batched SBS workload.

Workload ("sbs-batched-16view", the config the metric is quoted on): SDF of a
seeded smooth union (k=0.05) of 48 spheres and 16 rounded boxes, sampled at
octree depth 7 with 8-voxel bricks (1024^3 effective grid), DX layout 4 bytes
per value (213,585 bricks, 623 MB); 16 views of uneven size (512..2048 per side,
33.6 Mrays) on a radius-3 orbit, rendered in one persistent launch per step with
the reference NEWTON finder, NORMAL mode, closest hit.  A step renders all 16
views into a device hit buffer (t, primId, normal; 16 B per ray).

Arms: default = this engine (CUDA, sm_103a); --impl reference = the reference's
CPU algorithm for the same path (the oracle port in oracle/, OpenMP over all host
cores) on a bounded pixel sample of the same workload.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "SBS Mrays/s (plain finder, 16-view batched persistent launch)"
UNIT = "Mrays/s"
L2_FLUSH_BYTES = 256 << 20


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=60)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--depth", type=int, default=7)
    ap.add_argument("--brick", type=int, default=8)
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="target CPU time of the baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--variant", type=int, default=0,
                    help="render kernel: 0 per-lane rays, 1 warp packet, 2 per-lane rays with refill")
    ap.add_argument("--refill", type=int, default=8, help="variant 2: idle lanes that trigger a refill")
    ap.add_argument("--block-warps", type=int, default=4)
    ap.add_argument("--stage", type=int, default=0, help="packet kernel: stage bricks in shared memory")
    ap.add_argument("--tile-w", type=int, default=8, choices=(4, 8, 16, 32), help="warp pixel tile width (no autotune)")
    ap.add_argument("--stack", type=int, default=64, choices=(32, 64), help="traversal stack entries (no autotune)")
    ap.add_argument("--no-dr", action="store_true", help="skip the differentiable-render measurement")
    ap.add_argument("--dr-iters", type=int, default=200, help="reconstruction iterations (the first 10 untimed)")
    ap.add_argument("--dr-aggregate", type=int, default=1, help="warp-aggregated gradient atomics")
    ap.add_argument("--only-dr", action="store_true", help="measure the differentiable render alone (profiling)")
    ap.add_argument("--no-configs", action="store_true", help="skip the sphere and triangle-mesh lines")
    ap.add_argument("--no-autotune", action="store_true", help="use --variant/--block-warps/--stage as given")
    ap.add_argument("--no-graph", action="store_true", help="launch directly instead of replaying a CUDA graph")
    ap.add_argument("--no-proposal", action="store_true", help="skip the learned-proposal measurement")
    ap.add_argument("--no-device-bvh", action="store_true", help="skip the device BVH build measurement")
    ap.add_argument("--fma", type=int, default=1, choices=(0, 1),
                    help="headline kernel: 1 = compiled with FP contraction (within the forward parity tolerance), "
                         "0 = bit-exact; the other one is timed beside it")
    ap.add_argument("--prop-steps", type=int, default=20000, help="proposal training steps (batch 8192)")
    ap.add_argument("--prop-train-views", type=int, default=64, help="proposal training views (1024^2 each)")
    return ap.parse_args()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 100 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.dev = device_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax = float(p[2])
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def job_rate(ms_local, rays_per_rank, world, device=None):
    """Whole-job throughput of `world` replicas: the slowest rank's time (MAX
    all-reduce over the process group when world > 1) and the rays of all ranks
    over it.  Returns (ms, Mrays/s)."""
    ms = float(ms_local)
    if world > 1:
        import torch
        t = torch.tensor([ms], dtype=torch.float64, device=device)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    return ms, world * rays_per_rank / (ms * 1e-3) / 1e6


def build_workload(args):
    from litert_gb300 import lrt, scenes
    t0 = time.time()
    h, nodes, values = lrt.sbs_from_sdf(scenes.union_sdf(), args.depth, args.brick)
    views = scenes.union_views()
    return h, nodes, values, views, time.time() - t0


def gpu_build(args, host):
    """The same scene from the GPU builder: wall time (after one warm-up build)
    and whether it equals the host builder's output."""
    from litert_gb300 import lrt, scenes
    lrt.sbs_from_sdf(scenes.union_sdf(), 4, args.brick, gpu=0)   # context and module load
    t0 = time.time()
    h, nodes, values = lrt.sbs_from_sdf(scenes.union_sdf(), args.depth, args.brick, gpu=0)
    dt = time.time() - t0
    same = bool(np.array_equal(nodes, host[1]) and np.array_equal(values, host[2]))
    return dt, same


def run_device_bvh(args, h, nodes, values, views, tuned, hits, flush, stream, torch):
    """Scene commit wall time with the host binned-SAH BVH, the device SAH build
    (the same tree) and the device linear BVH (second commit of each, after a
    warm-up commit), and the headline render through each device-built tree with
    the same launch shape, timed like the headline (CUDA events, L2 flush between
    steps)."""
    from litert_gb300 import lrt
    out = {}
    n_rays = sum(w * hh for w, hh, _, _ in views)
    for builder, name in ((0, "host_sah"), (1, "device_sah"), (2, "device_lbvh")):
        s = lrt.Scene(0)
        s.set_tuning("bvh_builder", builder)
        gid = s.add_sbs(h, nodes, values)
        s.add_instance(gid)
        s.commit_scene()
        t0 = time.perf_counter()
        s.commit_scene()
        out["commit_s_" + name] = round(time.perf_counter() - t0, 3)
        if builder == 0:
            s.close()
            continue
        s.set_preset(render_mode=lrt.RENDER_MODE_NORMAL, sdf_node_intersect=lrt.INTERSECT_NEWTON)
        s.set_tuning("fma", args.fma)
        if tuned:
            for k in ("variant", "block_warps", "stage", "tile_w", "stack"):
                s.set_tuning(k, tuned[k])
        g = s.graph_create(views, hits_ptr=hits.data_ptr())
        for _ in range(args.warmup):
            flush.fill_(1.0)
            s.graph_launch(g, stream.cuda_stream)
        ts = []
        for i in range(args.steps):
            flush.fill_(float(i))
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            s.graph_launch(g, stream.cuda_stream)
            b.record(stream)
            b.synchronize()
            ts.append(a.elapsed_time(b))
        lrt.Scene.graph_destroy(g)
        s.close()
        ms = sum(ts) / len(ts)
        out["render_value_" + name] = n_rays / (ms * 1e-3) / 1e6
    return out


def cpu_sample(views, n_target, seed=0):
    """An evenly spaced pixel sample over all views: list of (view index, pixel
    ids).  Pixel i * (w * h) // k for i < k (every pixel when k = w * h), so the
    sample's counters do not drift with its size (a whole-number stride cut to
    k pixels would keep only the top rows of each view)."""
    total = sum(w * h for w, h, _, _ in views)
    out = []
    for vi, (w, h, _, _) in enumerate(views):
        n = w * h
        k = min(n, max(1, int(round(n_target * n / total))))
        idx = (np.arange(k, dtype=np.uint64) * np.uint64(n)) // np.uint64(k)
        idx = np.minimum(idx + np.uint64(seed % max(1, n // k)), np.uint64(n - 1))
        out.append((vi, idx.astype(np.uint32)))
    return out


def run_cpu_baseline(h, nodes, values, views, pairs, seconds, closest_hit=True):
    """Oracle port of the reference CPU path, all host threads, bounded sample.
    closest_hit=False walks the BVH2 as the reference's BVH2TraverseF32 does
    (stop at the first SDF leaf that hits); True returns the closest hit, the
    engine's result, whose counters give the engine's algorithmic bytes."""
    from litert_gb300 import lrt
    from oracle import oracle as orc
    osc = orc.Scene("sbs", sbs=(orc.SbsHeader(h.brick_size, h.brick_pad, h.bytes_per_value, h.aux_data), nodes, values),
                    pairs=pairs, intersect=2, render_mode=8, closest_hit=closest_hit)
    cores = os.cpu_count() or 1

    def run(n):
        cnt_tot = np.zeros(6)
        t0 = time.perf_counter()
        rays = 0
        for vi, pix in cpu_sample(views, n):
            w, hh, wv, pj = views[vi]
            _, cnt = osc.render_pixels(w, hh, lrt.inverse4x4(pj), lrt.inverse4x4(wv), pix, threads=cores)
            cnt_tot += [cnt.n_fat, cnt.n_leaf, cnt.n_vox, cnt.n_vox_loaded, cnt.n_finder, cnt.n_tri]
            rays += pix.size
        return rays, time.perf_counter() - t0, cnt_tot

    r0, t0, _ = run(20000)
    total = sum(w * hh for w, hh, _, _ in views)
    n = int(min(total, max(20000, 20000 * seconds / max(t0, 1e-3))))
    rays, dt, cnt = run(n)
    return dict(value=rays / dt / 1e6, rays=rays, seconds=dt, cores=cores, counters=cnt)


def run_small_configs(args, dev, torch):
    """The other primary-ray configurations, device-timed like the headline:
    sphere SBS (64^3 effective: depth 4, 4-voxel bricks; one 256^2 view and the
    same view replicated 16x in one launch) and the displaced icosphere mesh
    (327,680 triangles, 1920x1080).  Each with its oracle-port CPU rate."""
    from litert_gb300 import lrt, scenes
    from oracle import oracle as orc
    out = []
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)

    def timed(scene, views, steps):
        n = sum(w * h for w, h, _, _ in views)
        hits = torch.empty(n * 4, dtype=torch.float32, device=dev)
        va = lrt.make_views(views)
        for _ in range(3):
            scene.render_device(va, len(views), hits_ptr=hits.data_ptr(), stream=stream.cuda_stream)
        torch.cuda.synchronize(dev)
        ts = []
        for i in range(steps):
            flush.fill_(float(i))
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            scene.render_device(va, len(views), hits_ptr=hits.data_ptr(), stream=stream.cuda_stream)
            b.record(stream)
            b.synchronize()
            ts.append(a.elapsed_time(b))
        ms = statistics.median(ts)
        return n, ms, n / (ms * 1e-3) / 1e6

    def cpu_rate(osc, views, threads=None):
        cores = threads or os.cpu_count() or 1
        t0 = time.perf_counter()
        rays = 0
        for w, h, wv, pj in views[:1]:
            osc.render(w, h, lrt.inverse4x4(pj), lrt.inverse4x4(wv), threads=cores)
            rays += w * h
        return rays / (time.perf_counter() - t0) / 1e6, cores

    # config 1: sphere
    h, nodes, values = lrt.sbs_from_sdf(scenes.sphere_sdf(), 4, 4)
    sc = lrt.Scene(dev.index)
    g = sc.add_sbs(h, nodes, values)
    sc.add_instance(g)
    sc.commit_scene()
    sc.set_preset(render_mode=lrt.RENDER_MODE_NORMAL, sdf_node_intersect=lrt.INTERSECT_NEWTON)
    v1 = [scenes.sphere_view(256, 256)]
    osc = orc.Scene("sbs", sbs=(orc.SbsHeader(h.brick_size, h.brick_pad, h.bytes_per_value, h.aux_data), nodes, values),
                    intersect=2, render_mode=8)
    cpu, cores = cpu_rate(osc, v1)
    cpu1, _ = cpu_rate(osc, v1, threads=1)   # the reference's Render path is single-threaded
    for name, views in (("sphere-sbs-256", v1), ("sphere-sbs-256-x16", v1 * 16)):
        n, ms, mr = timed(sc, views, max(args.steps, 10))
        out.append({"workload": name, "value": mr, "unit": UNIT, "ms_per_step": ms, "rays_per_step": n,
                    "bricks": int(nodes.shape[0]),
                    "cpu_baseline": {"value": cpu, "unit": UNIT, "cores": cores, "kind": "port",
                                     "sample": "the 256x256 view"},
                    "cpu_single_thread": {"value": cpu1, "unit": UNIT, "cores": 1, "kind": "port",
                                          "sample": "the 256x256 view"}})
    sc.close()
    # config 2: triangles
    verts, faces = scenes.displaced_icosphere(subdiv=7)
    sc = lrt.Scene(dev.index)
    g = sc.add_triangles(verts, faces)
    sc.add_instance(g)
    sc.commit_scene()
    sc.set_preset(render_mode=lrt.RENDER_MODE_NORMAL)
    v2 = [scenes.mesh_view()]
    n, ms, mr = timed(sc, v2, max(args.steps, 10))
    osc = orc.Scene("mesh", mesh=(verts, faces), render_mode=8)
    cpu, cores = cpu_rate(osc, v2)
    out.append({"workload": "icosphere-327k-1920x1080", "value": mr, "unit": UNIT, "ms_per_step": ms,
                "rays_per_step": n, "triangles": int(faces.shape[0]),
                "cpu_baseline": {"value": cpu, "unit": UNIT, "cores": cores, "kind": "port",
                                 "sample": "the 1920x1080 view"}})
    sc.close()
    return out


def run_proposal(args, scene, dev, torch):
    """Learned proposal on the large SBS scene: triples from 64 training views
    (1024^2, seed 6), Adam training (lr 1e-3, batch 8192, seed 7), then plain vs
    proposal Mrays/s on 16 held-out views (1024^2, seed 8), each as a replayed
    CUDA graph, with the hit records compared bit for bit."""
    from litert_gb300 import lrt, proposal as pp, scenes
    train_views = scenes.proposal_views(args.prop_train_views, 1024, seed=6)
    eval_views = scenes.proposal_views(16, 1024, seed=8)
    pp.set_weights(scene, pp.init_weights(7))
    pp.clear(scene)
    t0 = time.time()
    n_trip = pp.collect(scene, train_views, capacity=min(50_000_000, len(train_views) * (1 << 20)))
    t_collect = time.time() - t0
    t0 = time.time()
    losses = pp.train(scene, args.prop_steps, batch=8192, lr=1e-3, seed=7)
    t_train = time.time() - t0
    # batched inference over the collected triples on both tensor-core engines
    n_inf = int(min(n_trip, 8 << 20))
    infer = {"samples": n_inf}
    if n_inf:
        ys = {}
        for name, eng in (("mma_sync", pp.ENGINE_MMA), ("tcgen05", pp.ENGINE_TCGEN05)):
            pp.infer(scene, 0, n_inf, engine=eng, timed=True)
            y, t_ms = pp.infer(scene, 0, n_inf, engine=eng, timed=True)
            ys[name] = y
            infer[name + "_ms"] = t_ms
            infer[name + "_gsamples_s"] = n_inf / (t_ms * 1e-3) / 1e9
        infer["max_abs_diff"] = float(np.abs(ys["mma_sync"] - ys["tcgen05"]).max())
    n = sum(w * h for w, h, _, _ in eval_views)
    hits = torch.empty(n * 4, dtype=torch.float32, device=dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    out = {}
    recs = {}
    stats = {}
    trained_w = pp.get_weights(scene)
    scene.set_tuning("fma", 0)   # the proposal kernel is compiled without contraction: compare like with like
    # plain; the proposal with the untrained (initial) network; the proposal with the trained one
    for name, mode, w in (("plain", 0, None), ("untrained", 1, pp.init_weights(7)), ("proposal", 1, trained_w)):
        if w is not None:
            pp.set_weights(scene, w)
        scene.set_tuning("proposal", mode)
        g = scene.graph_create(eval_views, hits_ptr=hits.data_ptr())
        for _ in range(3):
            scene.graph_launch(g, stream.cuda_stream)
        torch.cuda.synchronize(dev)
        if mode:
            pp.stats(scene)
        ts = []
        for i in range(max(args.steps, 5)):
            flush.fill_(float(i))
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            scene.graph_launch(g, stream.cuda_stream)
            b.record(stream)
            b.synchronize()
            ts.append(a.elapsed_time(b))
        if mode:
            stats[name] = pp.stats(scene)
        lrt.Scene.graph_destroy(g)
        ms = statistics.median(ts)
        out[name] = {"ms": ms, "mrays": n / (ms * 1e-3) / 1e6}
        recs[name] = hits.cpu().numpy().view(np.uint32).reshape(-1, 4).copy()
    # the same with the network trained on the other target: the first voxel the
    # walk runs the finder in (where a certified jump should land)
    scene.set_tuning("proposal", 0)
    scene.set_tuning("proposal_target", 1)
    pp.set_weights(scene, pp.init_weights(7))
    pp.clear(scene)
    pp.collect(scene, train_views, capacity=min(50_000_000, len(train_views) * (1 << 20)))
    losses_ff = pp.train(scene, args.prop_steps, batch=8192, lr=1e-3, seed=7)
    scene.set_tuning("proposal_target", 0)
    scene.set_tuning("proposal", 1)
    g = scene.graph_create(eval_views, hits_ptr=hits.data_ptr())
    for _ in range(3):
        scene.graph_launch(g, stream.cuda_stream)
    torch.cuda.synchronize(dev)
    pp.stats(scene)
    ts = []
    for i in range(max(args.steps, 5)):
        flush.fill_(float(i))
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        scene.graph_launch(g, stream.cuda_stream)
        b.record(stream)
        b.synchronize()
        ts.append(a.elapsed_time(b))
    stats["first_finder"] = pp.stats(scene)
    lrt.Scene.graph_destroy(g)
    ms_ff = statistics.median(ts)
    out["first_finder"] = {"ms": ms_ff, "mrays": n / (ms_ff * 1e-3) / 1e6}
    recs["first_finder"] = hits.cpu().numpy().view(np.uint32).reshape(-1, 4).copy()
    scene.set_tuning("proposal", 0)
    scene.set_tuning("fma", args.fma)
    st = stats["proposal"]
    reps = max(args.steps, 5)

    def per_step(d):
        return {k: v // reps for k, v in d.items()}
    # per-ray work of the plain walk (lrt_render_counters) and what the proposal removes from it
    cnt = scene.render_counters(eval_views).astype(np.float64) / n
    counters = {"plain_per_ray": {"nodes": cnt[0], "bricks": cnt[1], "voxel_steps": cnt[2], "finder_calls": cnt[3]},
                "proposal_per_ray": {"bricks_proposed": st["proposals"] / reps / n, "jumps": st["jumps"] / reps / n,
                                     "voxel_steps_skipped": st["steps_skipped"] / reps / n,
                                     "voxel_steps": cnt[2] - st["steps_skipped"] / reps / n,
                                     "finder_calls": cnt[3]}}
    a, b = recs["plain"], recs["proposal"]
    mask_same = np.array_equal(a[:, 1] != lrt.MISS, b[:, 1] != lrt.MISS)
    both = (a[:, 1] != lrt.MISS) & (b[:, 1] != lrt.MISS)
    dt = np.abs(a[both, 0].view(np.float32) - b[both, 0].view(np.float32))
    return {"metric": "SBS Mrays/s plain vs proposal at equal depth error", "unit": UNIT,
            "plain": out["plain"]["mrays"], "proposal": out["proposal"]["mrays"],
            "speedup": out["proposal"]["mrays"] / out["plain"]["mrays"],
            "ms_plain": out["plain"]["ms"], "ms_proposal": out["proposal"]["ms"],
            "hit_mask_identical": bool(mask_same), "records_identical": bool(np.array_equal(a, b)),
            "max_dt_over_extent": float(dt.max() / 2.0) if dt.size else 0.0,
            "proposals_per_step": st["proposals"] // max(1, len(ts)), "acceptance": st["jumps"] / max(1, st["proposals"]),
            "jump_hit_rate": st["jump_hits"] / max(1, st["jumps"]),
            "trained": per_step(stats["proposal"]), "untrained": per_step(stats["untrained"]),
            "counters": counters,
            "untrained_mrays": out["untrained"]["mrays"],
            "first_finder_target": {"mrays": out["first_finder"]["mrays"],
                                    "speedup": out["first_finder"]["mrays"] / out["plain"]["mrays"],
                                    "records_identical": bool(np.array_equal(recs["plain"], recs["first_finder"])),
                                    "stats": per_step(stats["first_finder"]),
                                    "loss_first": float(losses_ff[:10].mean()), "loss_last": float(losses_ff[-100:].mean())},
            "untrained_records_identical": bool(np.array_equal(recs["plain"], recs["untrained"])),
            "triples": int(n_trip), "train_steps": args.prop_steps, "batch": 8192,
            "loss_first": float(losses[:10].mean()), "loss_last": float(losses[-100:].mean()),
            "collect_s": round(t_collect, 2), "train_s": round(t_train, 2), "inference": infer,
            "config": {"workload": "proposal-16view-1024", "rays_per_step": n, "eval_views": 16,
                       "train_views": len(train_views), "network": "16-32-32-1 ReLU, BF16 mma.sync m16n8k16, FP32 accumulation"}}


def dr_setup(dev_index=0):
    """Differentiable reconstruction workload: target images rendered by the DR
    forward from the 256^3 target grid; the 128^3 sphere-initialised grid to optimise."""
    from litert_gb300 import dr, scenes
    t0 = time.time()
    target, init, views = scenes.dr_workload()
    R = dr.MultiRendererDR(dev_index)
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
    return R, init, views, imgs, time.time() - t0


def dr_preset(aggregate=1):
    from litert_gb300 import dr
    # Lambert, colour + geometry, spp 1, border_spp 256, Adam lr 3e-3; the batch's
    # gradients are summed (the reference keeps only the last view's: same work)
    return dr.default_preset(opt_lr=3e-3, spp=1, border_spp=256, seed=1, accumulate_batch=1,
                             warp_aggregate=aggregate)


def run_dr_cpu(R, init, views, imgs, preset, seconds_hint=True):
    """The oracle port of RenderDR (all host threads) on one of the views: the CPU
    time of one reconstruction iteration is 8x that (Adam is negligible)."""
    from litert_gb300 import lrt
    from oracle import oracle as orc
    from oracle import oracle_dr as od
    hdr, nodes, values, params = init
    osc = od.DrScene(orc.SbsHeader(hdr.brick_size, hdr.brick_pad, hdr.bytes_per_value, hdr.aux_data), nodes, values,
                     params.size, pairs=R.bvh2())
    lights = [(preset.lights[i].type, np.array(preset.lights[i].dir[:], np.float32),
               np.array(preset.lights[i].color[:], np.float32)) for i in range(preset.n_lights)]
    op = od.make_preset(render_mode=preset.render_mode, reconstruction=preset.reconstruction_flags, spp=preset.spp,
                        border_spp=preset.border_spp, seed=preset.seed, lights=lights, lr=preset.opt_lr)
    w, h, wv, pj = views[0]
    ov = od.make_view(w, h, wv, pj, lrt.inverse4x4)
    cores = os.cpu_count() or 1
    t0 = time.perf_counter()
    osc.render(params, op, ov, imgs[0], threads=cores)
    dt = time.perf_counter() - t0
    return dict(ms_per_iter=dt * len(views) * 1e3, cores=cores, seconds=dt)


def run_dr(args, dev, torch):
    """Differentiable SDF reconstruction: ms per OptimizeFixedStructure iteration
    (8 views at 512^2: forward + adjoint + border integral + Adam), device-timed."""
    R, init, views, imgs, t_setup = dr_setup(dev.index)
    preset = dr_preset(args.dr_aggregate)
    R.SetPreset(preset)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    warm = min(10, max(3, args.dr_iters // 10))
    first_losses = R.step(0)
    for i in range(1, warm):
        R.step(i, want_losses=False)
    torch.cuda.synchronize(dev)
    n_timed = max(1, args.dr_iters - warm)
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(n_timed)]
    clocks = ClockSampler(dev.index)
    clocks.start()
    launches = 0
    e2e = []
    last_losses = first_losses
    for k in range(n_timed):
        flush.fill_(float(k))
        torch.cuda.synchronize(dev)
        # device time between the events; end to end (wall clock) the C-ABI step
        # with the per-view losses read back to the host, on the same iterations
        t0 = time.perf_counter()
        evs[k][0].record(stream)
        last_losses = R.step(warm + k)
        evs[k][1].record(stream)
        e2e.append((time.perf_counter() - t0) * 1e3)
        launches += R.last_launch_count()
    torch.cuda.synchronize(dev)
    clk = clocks.stop()
    times = sorted(a.elapsed_time(b) for a, b in evs)
    ms = statistics.median(times)
    out = {"metric": "DR backward ms/iter", "value": ms, "unit": "ms/iter", "higher_is_better": False,
           "mean_ms": sum(times) / len(times), "min_ms": times[0], "max_ms": times[-1],
           "iterations": warm + n_timed, "timed_iterations": n_timed, "gpu_launches": launches,
           "launches_per_iter": launches / n_timed,
           "e2e": {"value": statistics.median(e2e), "unit": "ms/iter", "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 8 * len(views)},
           "loss_first": float(np.mean(first_losses)), "loss_last": float(np.mean(last_losses)),
           "config": {"workload": "dr-reconstruction-8view", "views": len(views), "size": 512,
                      "target": "smooth-union grid 32^3 bricks x 8 voxels, position colours",
                      "optimised": "grid 32^3 bricks x 4 voxels (129^3 distances + 33^3 RGB)",
                      "params": int(init[3].size), "render_mode": "LAMBERT", "spp": 1, "border_spp": 256,
                      "adam_lr": 3e-3, "batch": "8 views summed", "warp_aggregate": args.dr_aggregate,
                      "l2": "256 MiB write between timed iterations", "setup_s": round(t_setup, 2)},
           "clocks": clk}
    # the iteration with random and with SVM border sampling, and with the ray-casting
    # mask, each from the same parameters (Adam restarted), iterations numbered on
    # from the timed run; device time, median of 10 after 3 warm-up iterations
    variants = {}
    saved = R.get(0)
    it0 = warm + n_timed
    for name, kw in (("random_border_sampling", {}), ("svm_border_sampling", dict(border_sampling=1)),
                     ("raycasting_mask", dict(raycasting_mask=1))):
        p2 = dr_preset(args.dr_aggregate)
        for k, v in kw.items():
            setattr(p2, k, v)
        R.set_params(saved)
        R.SetPreset(p2)
        for i in range(3):
            R.step(it0 + i, want_losses=False)
        ts = []
        for k in range(10):
            flush.fill_(float(k))
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            R.step(it0 + 3 + k, want_losses=False)
            b.record(stream)
            b.synchronize()
            ts.append(a.elapsed_time(b))
        variants[name + "_ms"] = statistics.median(ts)
    out["variants"] = variants
    R.set_params(saved)
    R.SetPreset(preset)
    if not args.no_cpu_baseline:
        cpu = run_dr_cpu(R, [init[0], init[1], init[2], R.get(0)], views, imgs, preset)
        out["cpu_baseline"] = {"value": cpu["ms_per_iter"], "unit": "ms/iter", "cores": cpu["cores"], "kind": "port",
                               "sample": f"RenderDR of 1 of the 8 views on the current parameters "
                                         f"({cpu['seconds']:.1f} s), x8"}
    R.close()
    return out


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank != 0:
            return 0
        h, nodes, values, views, tb = build_workload(args)
        from litert_gb300 import lrt
        from oracle import oracle as orc
        pairs = lrt.build_bvh2(orc.node_boxes(nodes), 1)
        per_step = []
        cores = os.cpu_count() or 1
        budget = max(2.0, 120.0 / max(1, args.steps + args.warmup))
        res = None
        for i in range(args.warmup + args.steps):
            res = run_cpu_baseline(h, nodes, values, views, pairs, budget, closest_hit=False)
            if i >= args.warmup:
                per_step.append(res["value"])
        v = statistics.median(per_step)
        line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 33.596325e6 / (v * 1e6) * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "impl": "reference",
                "config": {"workload": "sbs-batched-16view", "rays_per_step": 33596325, "depth": args.depth,
                           "brick": args.brick, "finder": "NEWTON", "sample_rays_per_step": res["rays"]},
                "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                                 "sample": f"{res['rays']} strided pixels of the 16 views per step, the "
                                           "reference's first-hit BVH2 walk (BVH2TraverseF32) in the oracle port"},
                "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return 0

    import torch
    if args.only_dr:
        print(json.dumps(run_dr(args, torch.device("cuda", 0), torch)))
        return 0
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    from litert_gb300 import lrt
    from oracle import oracle as orc

    h, nodes, values, views, t_build = build_workload(args)
    t_gbuild, gbuild_same = gpu_build(args, (h, nodes, values)) if world == 1 else (None, None)
    scene = lrt.Scene(local if world > 1 else 0)
    g = scene.add_sbs(h, nodes, values)
    scene.add_instance(g)
    scene.commit_scene()
    scene.set_preset(render_mode=lrt.RENDER_MODE_NORMAL, sdf_node_intersect=lrt.INTERSECT_NEWTON)
    scene.set_tuning("variant", args.variant)
    scene.set_tuning("block_warps", args.block_warps)
    scene.set_tuning("stage", args.stage)
    scene.set_tuning("refill", args.refill)
    scene.set_tuning("fma", args.fma)
    scene.set_tuning("tile_w", args.tile_w)
    scene.set_tuning("stack", args.stack)
    dev = torch.device("cuda", local if world > 1 else 0)
    n_rays = sum(w * hh for w, hh, _, _ in views)
    hits = torch.empty(n_rays * 4, dtype=torch.float32, device=dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    va = lrt.make_views(views)
    stream = torch.cuda.current_stream(dev)
    tuned, tried = None, []
    if not args.no_autotune:
        tuned, tried = scene.autotune(views, reps=3)
    graph = None if args.no_graph else scene.graph_create(views, hits_ptr=hits.data_ptr())

    def step():
        if graph is not None:
            scene.graph_launch(graph, stream.cuda_stream)
        else:
            scene.render_device(va, len(views), hits_ptr=hits.data_ptr(), stream=stream.cuda_stream)

    for _ in range(args.warmup):
        flush.fill_(1.0)
        step()
    torch.cuda.synchronize(dev)

    clocks = ClockSampler(dev.index)
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    clocks.start()
    launches = 0
    for i in range(args.steps):
        flush.fill_(float(i))            # L2 flush between timed steps, outside the events
        evs[i][0].record(stream)
        step()
        evs[i][1].record(stream)
        launches += scene.last_launch_count()
    torch.cuda.synchronize(dev)
    if world > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    times = [a.elapsed_time(b) for a, b in evs]
    ms, value = job_rate(sum(times) / len(times), n_rays, world, dev)

    # end to end through the C ABI with host buffers (views in, hit buffer out, pinned host memory)
    # (default: the kernel writes device memory and each finished chunk of tile rows is
    # copied while the rest renders; "host_copy" 0: the kernel writes the host buffer)
    host_hits = torch.empty(n_rays * 4, dtype=torch.float32, pin_memory=True)

    def e2e_rate():
        e2e_times = []
        for i in range(args.warmup + args.steps):
            torch.cuda.synchronize(dev)
            t0 = time.perf_counter()
            st = lrt.lib().lrt_render_host(scene._ctx, lrt.C.cast(va, lrt.C.c_void_p), len(views),
                                           lrt.C.c_void_p(host_hits.data_ptr()), None, None)
            if st != 0:
                raise RuntimeError("lrt_render_host failed: %d" % st)
            if i >= args.warmup:
                e2e_times.append(time.perf_counter() - t0)
        return job_rate(statistics.median(e2e_times) * 1e3, n_rays, world, dev)[1]

    e2e = e2e_rate()
    scene.set_tuning("host_copy", 0)
    e2e_direct = e2e_rate()
    scene.set_tuning("host_copy", 1)

    # the other floating-point form of the same kernel, same launch shape, timed the same way
    other_fp = None
    if world == 1:
        scene.set_tuning("fma", 1 - args.fma)
        g2 = scene.graph_create(views, hits_ptr=hits.data_ptr())
        for _ in range(args.warmup):
            flush.fill_(1.0)
            scene.graph_launch(g2, stream.cuda_stream)
        ts2 = []
        for i in range(args.steps):
            flush.fill_(float(i))
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            scene.graph_launch(g2, stream.cuda_stream)
            b.record(stream)
            b.synchronize()
            ts2.append(a.elapsed_time(b))
        lrt.Scene.graph_destroy(g2)
        scene.set_tuning("fma", args.fma)
        ms2 = sum(ts2) / len(ts2)
        other_fp = {"fma": 1 - args.fma, "ms": ms2, "value": n_rays / (ms2 * 1e-3) / 1e6}

    line = None
    if rank == 0:
        # algorithmic bytes per ray (64 B per BVH2 fat pair, 16 B per brick node, 32 B per voxel's
        # corners, 16 B per output record) counted by the oracle on a pixel sample with the
        # engine's SAH BVH2 in the reference layout
        pairs = lrt.build_bvh2(orc.node_boxes(nodes), 1)
        cpu = None
        if not args.no_cpu_baseline:
            cpu = run_cpu_baseline(h, nodes, values, views, pairs, args.cpu_seconds)
            c = cpu["counters"]
            b_ray = (64 * c[0] + 16 * c[1] + 32 * c[2]) / cpu["rays"] + 16
        else:
            b_ray = None
        peaks = {}
        try:
            peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        except OSError:
            pass
        peak = peaks.get("hbm_gbs", 6800.0)
        achieved = (b_ray * n_rays / (ms * 1e-3) / 1e9) if b_ray else None
        if other_fp is not None and b_ray:
            other_fp["roofline_frac"] = b_ray * n_rays / (other_fp["ms"] * 1e-3) / 1e9 / peak
        traffic = None
        tp = os.path.join(ROOT, "profiles", "render_kernel_fused_sbs_batched16.md" if args.fma
                          else "render_kernel_sbs_batched16.md")
        if os.path.exists(tp):   # dram read+write of one launch, from the committed ncu summary
            for ln in open(tp):
                if ln.startswith("traffic_bytes_per_launch:"):
                    traffic = int(ln.split(":")[1])
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": "sbs-batched-16view", "rays_per_step": n_rays, "views": len(views),
                       "depth": args.depth, "brick": args.brick, "bricks": int(nodes.shape[0]),
                       "brick_bytes": int(values.nbytes), "finder": "NEWTON", "render_mode": "NORMAL",
                       "l2": "256 MiB write between timed steps; scene data 623 MB > L2",
                       "scene_build_s": round(t_build, 2),
                       "scene_build_gpu_s": None if t_gbuild is None else round(t_gbuild, 3),
                       "scene_build_gpu_identical": gbuild_same, "parallelism": f"replicas{world}",
                       "launch": "CUDA graph replay" if graph is not None else "direct",
                       "tuning": tuned, "autotune_candidates": len(tried),
                       "fp": ("FP32 with contraction (FMA); forward parity tolerance" if args.fma
                              else "FP32 without contraction; bit-exact to the reference x86-64 build")},
            "other_fp": other_fp,
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(len(views) * 136),
                    "d2h_bytes_per_step": int(n_rays * 16),
                    "path": "lrt_render_host into page-locked memory: chunks of tile rows copied while the "
                            "render runs", "direct_host_writes": e2e_direct},
            "gpu_launches": launches,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                         "bytes_per_ray": b_ray,
                         "peak_source": "measured" if "hbm_gbs" in peaks else "fallback"},
            "clocks": clk,
        }
        if cpu:
            line["cpu_baseline"] = {"value": cpu["value"], "unit": UNIT, "cores": cpu["cores"], "kind": "port",
                                    "sample": f"{cpu['rays']} strided pixels of the 16 views ({cpu['seconds']:.1f} s)"}
        if not args.no_proposal and world == 1:
            line["proposal"] = run_proposal(args, scene, dev, torch)
        if not args.no_device_bvh and world == 1:
            line["device_bvh"] = run_device_bvh(args, h, nodes, values, views, tuned, hits, flush, stream, torch)
        if not args.no_dr and world == 1:
            line["dr"] = run_dr(args, dev, torch)
        if world == 1 and not args.no_configs:
            line["other_configs"] = run_small_configs(args, dev, torch)
        print(json.dumps(line))
    if graph is not None:
        lrt.Scene.graph_destroy(graph)
    scene.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
