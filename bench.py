"""Benchmark of the path-tracing core on the plain per-frame path.

Workload (one step = one render pass = one sample per pixel over the frame, the
per-pass contract of src/RendererCore.cpp:248-469): the glass-icosphere Cornell box
(81,954 triangles, SAH BVH with leaf <= 4), 1024x1024, NEE + MIS, roulette after bounce
3, at most 16 bounces; synthetic seeded scene, per-pass seeds from mt19937(0).

Printed (one JSON line on rank 0):
  value        Mrays/s over the timed passes: every traceRay-equivalent query (primary,
               extension, NEE shadow, MIS) / device time of the passes (CUDA events on the
               context stream), inputs resident in HBM, L2 flushed between passes
  e2e          the same metric through the C-ABI with host buffers: per pass the camera
               block goes host -> device and the tonemapped frame comes back
  roofline     the extend (closest-hit) kernel: algorithmic bytes (32 B per box test,
               48 B per triangle test, 52 B of ray/hit records per ray) / its event time,
               against the measured L2 read bandwidth (the node + triangle set, ~9 MB,
               stays in L2); hbm_frac against MEASURED_PEAKS.json's HBM copy bandwidth
  cpu_baseline the reference kernel source compiled as C++ (oracle/_ref), all host
               threads, on a band of rows of the same frame
`--impl reference` times that CPU reference alone on the same workload.
With torchrun (N > 1) every rank renders its own replica (the work does not exchange
data; multi-GPU is replicas only) and the value is the sum of the ranks' rays over the
slowest rank's time.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mrays/s"
PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=64)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="c1")
    ap.add_argument("--e2e-steps", type=int, default=8)
    ap.add_argument("--cpu-seconds", type=float, default=8.0)
    ap.add_argument("--no-cpu", action="store_true")
    # batched (c2) and served (c3) comparisons against the plain per-pass loop
    ap.add_argument("--jobs", type=int, default=64)
    ap.add_argument("--spp", type=int, default=4, help="c2: passes per job")
    ap.add_argument("--pool", type=int, default=0, help="batch path slots (0: 2M)")
    ap.add_argument("--requests", type=int, default=40)
    ap.add_argument("--rate", type=float, default=20.0, help="c3: Poisson arrival rate (req/s)")
    ap.add_argument("--res-max", type=int, default=1024)
    ap.add_argument("--spp-max", type=int, default=128)
    ap.add_argument("--max-tris", type=int, default=500_000)
    ap.add_argument("--profile", action="store_true", help="c2: per-kernel split of the batched run")
    ap.add_argument("--quality", default="", help="comma list of configs: RMSE against the FP64 references")
    ap.add_argument("--trace-bench", type=int, default=0, help="traversal alone on this many seeded rays")
    ap.add_argument("--tail", type=int, default=-1, help="paths left at which a pass ends in the tail kernel "
                                                         "(-1 auto, 0 off)")
    ap.add_argument("--tree", type=int, default=1,
                    help="interior hierarchy: 0 reference nodes, 1 binary SAH over the reference leaves, 2 four-wide")
    return ap.parse_args()


def dist_init(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        return rank, local, ws, dist
    return rank, local, ws, None


def peaks():
    try:
        with open(PEAKS_FILE) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


class Clocks:
    """nvidia-smi samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def scene_for(name):
    from yune_gb300 import scenes
    return scenes.CONFIGS[name]()


def cpu_reference(scene, seeds, seconds, want_rays=True):
    """Times the reference kernel source (compiled as C++) on bands of rows of the frame
    with all host threads; rays counted by the oracle on the same band (same algorithm,
    bit-identical results). Falls back to the oracle port when the compiled reference is
    not available."""
    from oracle import oracle_py as O
    W, H = scene.width, scene.height
    cfg = dict(scene.cfg)
    threads = os.cpu_count() or 1
    use_ref = O.ref() is not None
    kind = "reference" if use_ref else "port"
    note = ""
    if use_ref and (cfg.get("brdf_model", 0) or cfg.get("mis_lobe_fix", 0)):
        # udpt.cl has neither the Oren-Nayar term nor the lobe fix: it runs its nearest
        # variant (Lambert, reference MIS), and the oracle counts the rays of that variant
        cfg["brdf_model"] = 0
        cfg["mis_lobe_fix"] = 0
        note = "; udpt.cl with -DMIS (Lambert diffuse, no lobe fix)"
    acc = np.zeros((H, W, 4), np.float32)
    band = max(1, H // 64)
    rows_done, t_total, rays = 0, 0.0, 0
    y = 0
    k = 0
    while t_total < seconds and y < H:
        r = (y, min(H, y + band))
        t0 = time.perf_counter()
        if use_ref:
            O.ref_render(scene, acc, seeds[k % len(seeds)], 1, "udpt_mis" if cfg["mis"] else "udpt_a",
                         cfg["rr_threshold"], cfg["max_depth"], threads=threads, rows=r)
        else:
            c = O.render(scene, acc, seeds[k % len(seeds)], 1, cfg, threads=threads, rows=r)
        dt = time.perf_counter() - t0
        t_total += dt
        if use_ref and want_rays:
            acc2 = np.zeros_like(acc)
            c = O.render(scene, acc2, seeds[k % len(seeds)], 1, cfg, threads=threads, rows=r)
        rays += c["rays"]
        rows_done += r[1] - r[0]
        y = r[1]
    value = rays / t_total / 1e6 if t_total > 0 else 0.0
    return {"value": value, "unit": METRIC, "cores": threads, "kind": kind,
            "sample": "%d of %d rows x %d px, 1 pass, %.1f s%s" % (rows_done, H, W, t_total, note),
            "samples_per_s": rows_done * W / t_total if t_total > 0 else 0.0}


def run_reference(args, rank, ws, dist):
    scene = scene_for(args.config)
    from yune_gb300 import scenes
    seeds = scenes.pass_seeds(0, args.steps + args.warmup)
    if rank != 0:
        return
    cb = cpu_reference(scene, seeds, args.cpu_seconds)
    cfg = {"workload": "%s: %d tris, %dx%d, cfg %s" % (args.config, scene.n_tri, scene.width, scene.height,
                                                      json.dumps(scene.cfg, sort_keys=True)),
           "spp_total": scene.spp}
    line = {"metric": METRIC, "value": cb["value"], "unit": METRIC, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "fp32", "data": "synthetic", "config": cfg,
            "cpu_baseline": cb, "e2e": {"value": cb["value"], "unit": METRIC, "h2d_bytes_per_step": 0,
                                        "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_ours(args, rank, local, ws, dist):
    from yune_gb300 import quality, scenes
    from yune_gb300.core import Renderer
    scene = scene_for(args.config)
    seeds = scenes.pass_seeds(0, args.warmup + args.steps + args.e2e_steps)
    W, H = scene.width, scene.height
    r = Renderer(local)
    r.set_tree_mode(args.tree)
    r.set_tail_paths(args.tail)
    sid = r.upload(scene)
    r.set_camera(scene.cam)
    aid = r.alloc_accum(W, H)
    l2 = r.measure_l2_gbs(48 << 20, 20)
    # warm-up
    for k in range(args.warmup):
        r.render(sid, aid, seeds[k], reset=1 if k == 0 else 0, cfg=scene.cfg)
    r.synchronize()
    r.reset_stats()
    r.set_profiling(True)
    if dist:
        dist.barrier()
    ms_total = 0.0
    with Clocks(local) as clk:
        for k in range(args.steps):
            r.flush_l2(256 << 20)
            r.render(sid, aid, seeds[args.warmup + k], reset=0, cfg=scene.cfg)
            ms_total += r.last_pass_ms()
    r.synchronize()
    st = r.stats()
    kt = r.kernel_times()
    r.set_profiling(False)
    # e2e through the C-ABI with host buffers: camera in, tonemapped frame out
    ldr = None
    t0 = time.perf_counter()
    for k in range(args.e2e_steps):
        r.set_camera(scene.cam)
        r.render(sid, aid, seeds[args.warmup + args.steps + k], reset=0, cfg=scene.cfg)
        ldr = r.tonemap(aid)
    e2e_s = time.perf_counter() - t0
    e2e_stats = r.stats()
    e2e_rays = e2e_stats["rays"] - st["rays"]
    img = r.read_accum(aid)
    rays = st["rays"]
    t_s = ms_total / 1e3
    if dist:
        import torch
        tt = torch.tensor([t_s, float(rays), e2e_s, float(e2e_rays)], dtype=torch.float64)
        mx = tt.clone()
        dist.all_reduce(mx, op=dist.ReduceOp.MAX)
        sm = tt.clone()
        dist.all_reduce(sm, op=dist.ReduceOp.SUM)
        t_s, e2e_s = mx[0].item(), mx[2].item()
        rays, e2e_rays = sm[1].item(), sm[3].item()
    if rank != 0:
        r.close()
        return
    pk, pk_kind = peaks()
    ext_bytes = 32.0 * st["ext_boxes"] + 48.0 * st["ext_tris"] + 32.0 * st["ext_rays"] + 52.0 * st["ext_rays"]
    ext_ms = kt["extend_ms"]
    achieved = ext_bytes / (ext_ms / 1e3) / 1e9 if ext_ms > 0 else 0.0
    launches = int(kt["raygen_launches"] + kt["extend_launches"] + kt["occlusion_launches"] + kt["logic_launches"]
                   + kt["tail_launches"])
    traffic = None
    prof_file = os.path.join(ROOT, "profiles", "extend_traffic.json")
    if os.path.exists(prof_file):
        with open(prof_file) as f:
            tr = json.load(f)
        if tr.get("config") == args.config and kt["extend_launches"]:
            traffic = tr.get("dram_bytes_per_launch")
    samples = st["samples"]
    line = {
        "metric": METRIC, "value": rays / t_s / 1e6, "unit": METRIC, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_total / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32", "data": "synthetic (seeded procedural scene)",
        "config": {"workload": "%s: glass icosphere Cornell box, %d tris, %dx%d, 1 spp per step, NEE+MIS, RR after "
                               "bounce 3, max depth %d" % (args.config, scene.n_tri, W, H, scene.cfg["max_depth"]),
                   "spp_total": scene.spp, "l2": "flushed between timed steps (256 MB write)",
                   "parallelism": "replicas" if ws > 1 else "single GPU"},
        "samples_per_s": samples / t_s * (ws if dist else 1),
        "rays_per_sample": st["rays"] / max(1, samples),
        "traversed_rays": st["traversed"],
        "gpu_launches": launches,
        "kernel_ms": {"raygen": kt["raygen_ms"], "extend": kt["extend_ms"], "occlusion": kt["occlusion_ms"],
                      "logic": kt["logic_ms"], "tail": kt["tail_ms"], "rounds": kt["rounds"]},
        "roofline": {"kernel": "k_trace_paths<false> (extend)", "bound": "l2", "achieved": achieved,
                     "peak": l2, "unit": "GB/s", "frac": achieved / l2 if l2 else None, "traffic": traffic,
                     "peak_source": "measured L2 read bandwidth (yc_measure_l2_gbs, 48 MB x 20 sweeps)",
                     "hbm_peak": pk.get("hbm_gbs"), "hbm_frac": achieved / pk.get("hbm_gbs", 1.0),
                     "hbm_peak_source": pk_kind,
                     "bytes_per_ray": ext_bytes / max(1, st["ext_rays"]),
                     "box_tests_per_ray": st["ext_boxes"] / max(1, st["ext_rays"]),
                     "tri_tests_per_ray": st["ext_tris"] / max(1, st["ext_rays"])},
        "e2e": {"value": e2e_rays / e2e_s / 1e6 if e2e_s > 0 else 0.0, "unit": METRIC,
                "h2d_bytes_per_step": 80 + 4, "d2h_bytes_per_step": W * H * 16,
                "steps": args.e2e_steps},
        "clocks": clk.summary(),
        "image_error": quality.report(img, args.config, int(img[0, 0, 3])),
        "stack_overflow": st["stack_overflow"],
        "image_mean": float(np.nanmean(img[..., :3])),
    }
    if not args.no_cpu:
        line["cpu_baseline"] = cpu_reference(scene, seeds, args.cpu_seconds)
    r.close()
    print(json.dumps(line))


def run_c2(args):
    """Mixed batch: every job rendered pass by pass (plain) and all jobs in one batch."""
    from yune_gb300 import autotune, scenes, workloads
    from yune_gb300.batch import Batch
    from yune_gb300.core import Renderer
    jobs = workloads.c2_jobs(n_jobs=args.jobs, spp=args.spp, max_tris=args.max_tris)
    r = Renderer(0)
    r.set_tree_mode(args.tree)
    sids = [r.upload(s) for s in jobs]
    seeds = [scenes.pass_seeds(1000 + i, s.spp) for i, s in enumerate(jobs)]
    px = sum(s.width * s.height for s in jobs)
    out = {}
    # plain
    accs = [r.alloc_accum(s.width, s.height) for s in jobs]
    r.reset_stats()
    r.synchronize()
    t0 = time.perf_counter()
    for s, sid, a, sd in zip(jobs, sids, accs, seeds):
        r.set_camera(s.cam)
        r.render_passes(sid, a, sd, reset_first=1, cfg=s.cfg)
    r.synchronize()
    tp = time.perf_counter() - t0
    stp = r.stats()
    plain_imgs = [r.read_accum(a) for a in accs[:4]]
    for a in accs:
        r.free_accum(a)
    # batched: launch shape from the autotuner (untimed), unless --pool fixes the pool
    cap = max(r.scene_depth(sid) for sid in sids) + 2
    if args.pool:
        shape, trials, tune_s = autotune.BatchShape(pool_paths=args.pool), [], 0.0
    else:
        shape, trials, tune_s = autotune.tune_scenes(r, jobs, sids, stack_cap=cap)
    if args.profile:   # per-kernel split of the batched run (graph off, CUDA events per launch)
        accs = [r.alloc_accum(s.width, s.height) for s in jobs]
        b = Batch(r, use_graph=False, stack_cap=cap, **shape.kwargs())
        for s, sid, a, sd in zip(jobs, sids, accs, seeds):
            b.add_job(sid, a, s.cam, sd, s.cfg)
        r.set_profiling(True)
        b.run()
        kt_batch = r.kernel_times()
        r.set_profiling(False)
        b.close()
        for a in accs:
            r.free_accum(a)
    accs = [r.alloc_accum(s.width, s.height) for s in jobs]
    b = Batch(r, stack_cap=cap, **shape.kwargs())
    for s, sid, a, sd in zip(jobs, sids, accs, seeds):
        b.add_job(sid, a, s.cam, sd, s.cfg)
    r.reset_stats()
    r.synchronize()
    t0 = time.perf_counter()
    left = b.run()
    r.synchronize()
    tb = time.perf_counter() - t0
    stb = r.stats()
    same = all(np.array_equal(r.read_accum(a).view(np.int32), w.view(np.int32)) for a, w in zip(accs[:4], plain_imgs))
    b.close()
    out = {"metric": METRIC, "unit": METRIC, "config": {"workload": "c2 mixed batch", "jobs": len(jobs), "spp": args.spp,
                                                         "pixels_per_pass": px,
                                                         "triangles": int(sum(s.n_tri for s in jobs))},
           "plain": {"value": stp["rays"] / tp / 1e6, "seconds": tp, "samples_per_s": stp["samples"] / tp},
           "batched": {"value": stb["rays"] / tb / 1e6, "seconds": tb, "samples_per_s": stb["samples"] / tb,
                       "unfinished": left},
           "speedup": tp / tb, "equal_results": bool(same), "rays_equal": stp["rays"] == stb["rays"],
           "autotune": {"shape": shape.kwargs(), "seconds": tune_s,
                        "trials": [[t.kwargs(), ms] for t, ms in trials]}}
    if args.profile:
        out["batched"]["kernel_ms"] = kt_batch
    r.close()
    print(json.dumps(out))


def run_c3(args):
    """Served requests (continuous batching) against the plain first-come loop."""
    from yune_gb300 import serve, workloads
    from yune_gb300.core import Renderer
    resident = workloads.c3_scenes(8, max_tris=args.max_tris)
    reqs = workloads.c3_requests(args.requests, args.rate, len(resident), res_range=(256, args.res_max),
                                 spp_range=(16, args.spp_max))
    mk = lambda: [serve.Request(a, sc, w, h, spp, seed=i) for i, (a, sc, w, h, spp) in enumerate(reqs)]  # noqa: E731
    r = Renderer(0)
    r.reset_stats()
    srv = serve.Server(r, resident, hbm_budget=40 << 30, pool_paths=args.pool or (1 << 21))
    t0 = time.perf_counter()
    served = srv.run(mk())
    ts = time.perf_counter() - t0
    sts = r.stats()
    srv.close()
    r.reset_stats()
    t0 = time.perf_counter()
    plain = serve.serve_plain(r, resident, mk())
    tpl = time.perf_counter() - t0
    stp = r.stats()
    p50s, p99s = serve.percentiles(served)
    p50p, p99p = serve.percentiles(plain)
    out = {"metric": "p50/p99 time to target spp (s)", "unit": "s",
           "config": {"workload": "c3 serving", "requests": len(reqs), "rate_per_s": args.rate,
                      "resolution": [256, args.res_max], "spp": [16, args.spp_max],
                      "scene_triangles": [int(s.n_tri) for s in resident]},
           "served": {"p50": p50s, "p99": p99s, "Mrays_s": sts["rays"] / ts / 1e6, "seconds": ts},
           "plain": {"p50": p50p, "p99": p99p, "Mrays_s": stp["rays"] / tpl / 1e6, "seconds": tpl}}
    r.close()
    print(json.dumps(out))


def run_quality(args):
    """Relative RMSE of each configuration against its FP64 reference, at the
    configuration's passes and at four times as many (an unbiased estimator halves it)."""
    from yune_gb300 import quality, scenes
    from yune_gb300.core import Renderer
    r = Renderer(0)
    out = {"metric": "relative RMSE vs the 65,536-pass FP64 reference", "configs": {}}
    for name in args.quality.split(","):
        s = scenes.CONFIGS[name]()
        sid = r.upload(s)
        r.set_camera(s.cam)
        aid = r.alloc_accum(s.width, s.height)
        res = {}
        seeds = scenes.pass_seeds(11, 4 * s.spp)
        t0 = time.perf_counter()
        done = 0
        for n in (s.spp, 4 * s.spp):
            r.render_passes(sid, aid, seeds[done:n], reset_first=1 if done == 0 else 0, cfg=s.cfg)
            done = n
            res[str(n)] = quality.report(r.read_accum(aid), name, n)
        res["seconds"] = time.perf_counter() - t0
        a, b = res[str(s.spp)]["rel_rmse"], res[str(4 * s.spp)]["rel_rmse"]
        res["decay_ratio_4x"] = a / b if b > 0 else None
        a, b = res[str(s.spp)]["rmse_trimmed_1pct"], res[str(4 * s.spp)]["rmse_trimmed_1pct"]
        res["decay_ratio_4x_trimmed"] = a / b if b > 0 else None
        out["configs"][name] = res
        r.free_accum(aid)
        r.release(sid)
    r.close()
    print(json.dumps(out))


def run_trace_bench(args):
    """Traversal alone: seeded incoherent rays (origins uniform in the Cornell box,
    directions uniform on the sphere) through yc_trace_device, closest hit and any hit,
    inputs resident on the device, CUDA-event time of the trace kernel."""
    import torch
    from yune_gb300 import scenes
    from yune_gb300.core import Renderer
    scene = scene_for(args.config)
    n = args.trace_bench
    rays = torch.from_numpy(scenes.box_rays(n, seed=3)).cuda()
    tri = torch.empty(n, dtype=torch.int32, device="cuda")
    t = torch.empty(n, dtype=torch.float32, device="cuda")
    r = Renderer(0)
    r.set_tree_mode(args.tree)
    sid = r.upload(scene)
    out = {"metric": "traversal Mrays/s", "config": {"workload": "%s, %d seeded incoherent rays" % (args.config, n),
                                                     "tree_mode": args.tree}}
    for any_hit in (False, True):
        for _ in range(args.warmup):
            r.trace_device(sid, rays.data_ptr(), n, any_hit, tri.data_ptr(), t.data_ptr())
        r.synchronize()
        r.reset_stats()
        r.set_profiling(True)
        for _ in range(args.steps):
            r.flush_l2(256 << 20)
            r.trace_device(sid, rays.data_ptr(), n, any_hit, tri.data_ptr(), t.data_ptr())
        kt = r.kernel_times()
        r.set_profiling(False)
        st = r.stats()
        ms = kt["occlusion_ms"] if any_hit else kt["extend_ms"]
        pre = "any" if any_hit else "ext"
        nr = st[pre + "_rays"]
        nb = 32.0 * st[pre + "_boxes"] + 48.0 * st[pre + "_tris"] + (52.0 if not any_hit else 36.0) * nr
        out["any_hit" if any_hit else "closest"] = {
            "Mrays_s": nr / (ms / 1e3) / 1e6, "ms_per_launch": ms / args.steps,
            "box_tests_per_ray": st[pre + "_boxes"] / max(1, nr), "tri_tests_per_ray": st[pre + "_tris"] / max(1, nr),
            "algorithmic_GBs": nb / (ms / 1e3) / 1e9}
    r.close()
    print(json.dumps(out))


def main():
    args = parse()
    if args.quality:
        return run_quality(args)
    if args.trace_bench:
        return run_trace_bench(args)
    if args.impl == "ours" and args.config == "c2":
        return run_c2(args)
    if args.impl == "ours" and args.config == "c3":
        return run_c3(args)
    rank, local, ws, dist = dist_init(args)
    if args.impl == "reference":
        run_reference(args, rank, ws, dist)
    else:
        run_ours(args, rank, local, ws, dist)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
