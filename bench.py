"""Benchmark of the path-tracing core.

Default workload (--config c2, the mixed workload the batched/served target is stated on):
64 seeded scenes, each a Cornell box plus displaced icospheres (triangle totals
log-uniform in [1k, 500k], 6.44M in all), materials drawn from {Oren-Nayar, modified
Phong, dielectric}, resolutions drawn from {256^2, 512^2, 1280x720, 1920x1080} (59.6M
pixels per pass), NEE + MIS with udpt-primitives.cl's Oren-Nayar rule, roulette after
bounce 3, at most 16 bounces, no lobe fix (the reference's own MIS arithmetic, so the
CPU reference runs the same configuration). One step = one pass (one sample per pixel)
of every job of the mix; the configuration's 64 spp are 64 steps.

Printed (one JSON line on rank 0):
  value        Mrays/s of the batched form: the K timed passes of all 64 jobs rendered
               in one persistent wavefront (yc_batch_*); every traceRay-equivalent query
               (primary, extension, NEE shadow, MIS) over the CUDA-event time of the
               run, inputs resident in HBM; the median of --reps repetitions
  plain        the same passes through the plain one-frame-at-a-time path
               (yc_render_passes, job after job), timed the same way; its median, and
               batched_over_plain = the median of the per-repetition ratios
  equal_results every accumulator of the batched form equal bit for bit to the plain one
  walked_grays_per_s, samples_per_s  rays that walked a BVH, and pixel paths, per second
  roofline     the traversal kernel of the batched form (profiled copy): algorithmic
               bytes (32 B per box test, 48 B per triangle test, 84 B of ray and hit
               records per ray) over its event time, against the measured L2 read
               bandwidth; hbm_frac against MEASURED_PEAKS.json's HBM copy bandwidth
  e2e          the metric through the C-ABI with host buffers: per step every job's
               camera and pass seeds go host -> device (yc_batch_add_job), the batch runs
               and every job's tonemapped frame comes back (yc_tonemap); e2e_plain does
               the same with yc_set_camera + yc_render_passes
  cpu_baseline the reference kernel source (udpt.cl -DMIS with udpt-primitives.cl's
               Oren-Nayar rule) compiled as C++ (oracle/_ref), all host threads, on bands
               of rows of 8 of the 64 scenes (every eighth), each given time in proportion
               to its pixels
`--impl reference` times that CPU reference alone on the same workload; it generates
the scenes with the oracle library's copy of the scene producers and builds their BVHs
with the reference's own BVH::createBVH, so it loads no product library.
With torchrun (N > 1) every rank renders its own replica (the work does not exchange
data; multi-GPU is replicas only) and the value is the sum of the ranks' rays over the
slowest rank's time.
Other modes: --config c1 / c0 (one frame, batch engine against yc_render_pass), c4,
c0_bdpt, c4_mis, c0_bdpt_mis (per-pass BDPT), --config c3 (serving), --quality (RMSE
against the FP64 references), --trace-bench N (traversal alone).
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
L2_BYTES = 126 << 20   # GB300 L2 as the CUDA runtime reports it
PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="c2")
    ap.add_argument("--reps", type=int, default=3, help="c2: timed repetitions (median reported)")
    ap.add_argument("--e2e-steps", type=int, default=0, help="e2e steps (0: 8 for one frame, 2 for the mix)")
    ap.add_argument("--e2e-passes", type=int, default=0, help="passes per e2e step (0: 8 for one frame, 4 for "
                                                                 "the mix)")
    ap.add_argument("--groups", type=int, default=2, help="slot groups of the engine (c1 whole-job run)")
    ap.add_argument("--cpu-seconds", type=float, default=0.0, help="CPU baseline budget (0: 8 s, 16 s for the mix)")
    ap.add_argument("--no-cpu", action="store_true")
    # batched (c2) and served (c3) comparisons against the plain per-pass loop
    ap.add_argument("--jobs", type=int, default=64)
    ap.add_argument("--sample-every", type=int, default=8, help="c2 CPU baseline: every n-th job of the mix")
    ap.add_argument("--pool", type=int, default=0, help="batch path slots (0: 2M)")
    ap.add_argument("--shape", default="", help="c2: the batch's launch shape as JSON (BatchShape fields) instead "
                                                "of the autotuner's, e.g. to profile the tuned shape")
    ap.add_argument("--traffic-only", action="store_true",
                    help="c2: only two passes of every job through the batch engine (no graph), then print the "
                         "rays its traversal launches walked: the run an ncu capture of their DRAM bytes divides by")
    ap.add_argument("--requests", type=int, default=40)
    ap.add_argument("--rate", type=float, default=20.0, help="c3: Poisson arrival rate (req/s)")
    ap.add_argument("--rates", default="", help="c3: comma list of arrival rates to sweep (overrides --rate)")
    ap.add_argument("--hbm-budget-mb", type=int, default=40 << 10, help="c3: HBM budget of the accumulators in flight")
    ap.add_argument("--res-max", type=int, default=1024)
    ap.add_argument("--spp-max", type=int, default=128)
    ap.add_argument("--max-tris", type=int, default=500_000)
    ap.add_argument("--profile", action="store_true", help="c2: per-kernel split of the batched run")
    ap.add_argument("--quality", default="", help="comma list of configs: RMSE against the FP64 references")
    ap.add_argument("--trace-bench", type=int, default=0, help="traversal alone on this many seeded rays")
    ap.add_argument("--tail", type=int, default=-1, help="paths left at which a pass ends in the tail kernel "
                                                         "(-1 auto, 0 off)")
    ap.add_argument("--mixed", type=int, default=1,
                    help="1: a round's closest-hit and any-hit rays share one traversal launch; 0: one launch each")
    ap.add_argument("--ray-sort", type=int, default=32,
                    help="sort key of a round's rays: origin bits * 10 + direction bits per axis (0: queue order)")
    ap.add_argument("--ray-sort-min", type=int, default=65536, help="rounds with fewer rays are not sorted")
    ap.add_argument("--shade-sort-min", type=int, default=65536,
                    help="per-pass path: shade queues of at least this many paths are sorted (0: never)")
    ap.add_argument("--res", default="", help="c4: frame size WxH instead of 3840x2160 (profiling captures)")
    ap.add_argument("--stack-smem", type=int, default=0,
                    help="walk-stack entries the per-pass traversal keeps in shared memory (0: the default 12; "
                         "64: the whole stack)")
    ap.add_argument("--tree", type=int, default=1,
                    help="interior hierarchy: 0 reference nodes, 1 binary SAH over the reference leaves, 2 four-wide")
    a = ap.parse_args()
    mix = a.config == "c2"
    a.e2e_steps = a.e2e_steps or (2 if mix else 8)
    a.e2e_passes = a.e2e_passes or (4 if mix else 8)
    a.cpu_seconds = a.cpu_seconds or (16.0 if mix else 8.0)
    return a


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


def reference_variant(cfg):
    """The compiled reference variant (oracle/_ref) that runs configuration `cfg`, and a
    note; None when no variant of the reference has the configuration."""
    if cfg.get("integrator", 0) != 0:
        return None, ""
    if not cfg.get("mis", 0):
        return ("udpt_a", "; udpt.cl as shipped") if not cfg.get("brdf_model", 0) else (None, "")
    v = "udpt_mis_on" if cfg.get("brdf_model", 0) == 1 else "udpt_mis"
    note = ("; udpt.cl -DMIS with udpt-primitives.cl's Oren-Nayar rule" if v == "udpt_mis_on"
            else "; udpt.cl -DMIS")
    return v, note


def _cpu_measure(scene, seeds, seconds, want_rays=True, band=0):
    """Times the reference kernel source (compiled as C++) on bands of rows of the frame
    with all host threads; rays counted by the oracle on the same band (same algorithm,
    bit-identical results). Falls back to the oracle port when the compiled reference has
    no variant for the configuration. band = 0: H/64 rows per band from the top of the
    frame; band > 0: bands of that many rows spread over the frame (a stride coprime to
    its height). Returns rays, seconds, rows, kind and a note."""
    from oracle import oracle_py as O
    W, H = scene.width, scene.height
    cfg = dict(scene.cfg)
    bdpt = cfg.get("integrator", 0) == 1
    bdpt_mis = cfg.get("integrator", 0) == 2
    threads = os.cpu_count() or 1
    use_ref = O.ref() is not None and not bdpt_mis
    note = ""
    if bdpt_mis:   # no reference implementation exists: the CPU statement is the baseline
        kmax = int(cfg.get("bdpt_bounces", 20))
        note = "; bidirectional tracer with MIS (the CPU statement), paths <= %d segments, %d lights" % (
            kmax, len(scene.lights))
    elif bdpt:
        bounces = int(cfg.get("bdpt_bounces", 20))
        variant = {(20, 1): "bdpt20", (8, 1): "bdpt8", (8, 4): "bdpt8_l4"}.get((bounces, len(scene.lights)))
        if use_ref and variant is None:
            use_ref = False
        note = "; bdpt.cl, %d vertices per subpath, %d lights" % (bounces, len(scene.lights))
    elif use_ref:
        if cfg.get("mis_lobe_fix", 0):
            # the reference has no lobe fix: it runs its own MIS arithmetic, and the oracle
            # counts the rays of that arithmetic
            cfg["mis_lobe_fix"] = 0
            note = "; without the lobe fix (reference MIS)"
        variant, vnote = reference_variant(cfg)
        if variant is None or len(scene.lights) != 1:
            use_ref = False
        note = vnote + note
    kind = "reference" if use_ref else "port"
    acc = np.zeros((H, W, 4), np.float32)
    if band <= 0:
        band = max(1, H // 64)
        starts = list(range(0, H, band))
    else:
        nb = (H + band - 1) // band
        step = next(q for q in range(nb // 3 + 1, nb + 1) if np.gcd(q, nb) == 1) if nb > 2 else 1
        starts = [((i * step) % nb) * band for i in range(nb)]

    def one(k, r, a, ref):
        if bdpt_mis:
            return O.render_bdpt_mis(scene, a, seeds[k % len(seeds)], 1, kmax, cfg, threads=threads, rows=r)
        if bdpt:
            if ref:
                O.ref_render(scene, a, seeds[k % len(seeds)], 1, variant, 0, 0, threads=threads, rows=r)
                return None
            return O.render_bdpt(scene, a, seeds[k % len(seeds)], 1, bounces, threads=threads, rows=r)
        if ref:
            O.ref_render(scene, a, seeds[k % len(seeds)], 1, variant, cfg["rr_threshold"], cfg["max_depth"],
                         threads=threads, rows=r)
            return None
        return O.render(scene, a, seeds[k % len(seeds)], 1, cfg, threads=threads, rows=r)

    rows_done, t_total, rays = 0, 0.0, 0
    k = 0
    while t_total < seconds:   # bands in order, frame after frame (pass k + 1 wraps around)
        y = starts[k % len(starts)]
        r = (y, min(H, y + band))
        t0 = time.perf_counter()
        c = one(k, r, acc, use_ref)
        t_total += time.perf_counter() - t0
        if c is None and want_rays:   # the oracle counts the rays of the same band
            c = one(k, r, np.zeros_like(acc), False)
        rays += c["rays"] if c else 0
        rows_done += r[1] - r[0]
        k += 1
    return {"rays": rays, "seconds": t_total, "rows": rows_done, "pixels": rows_done * W, "kind": kind,
            "note": note, "threads": threads}


def cpu_reference(scene, seeds, seconds, want_rays=True, band=0):
    """The CPU baseline on one frame (see _cpu_measure)."""
    m = _cpu_measure(scene, seeds, seconds, want_rays, band)
    W, H, t = scene.width, scene.height, m["seconds"]
    return {"value": m["rays"] / t / 1e6 if t > 0 else 0.0, "unit": METRIC, "cores": m["threads"], "kind": m["kind"],
            "sample": "%d rows of %d x %d px (%.2f passes' worth), %.1f s%s" % (m["rows"], H, W, m["rows"] / H, t,
                                                                            m["note"]),
            "samples_per_s": m["pixels"] / t if t > 0 else 0.0}


def cpu_reference_mix(jobs, idx, seeds, seconds):
    """The CPU baseline on the mix: the sampled jobs `idx`, each timed for a share of
    `seconds` in proportion to its pixels; Mrays/s = all rays over all time."""
    px = np.array([jobs[i].width * jobs[i].height for i in range(len(jobs))], np.float64)
    rays = t = pix = 0.0
    kinds, notes = set(), set()
    for i in range(len(jobs)):
        m = _cpu_measure(jobs[i], seeds[i], seconds * px[i] / px.sum())
        rays += m["rays"]
        t += m["seconds"]
        pix += m["pixels"]
        kinds.add(m["kind"])
        notes.add(m["note"])
        threads = m["threads"]
    return {"value": rays / t / 1e6 if t > 0 else 0.0, "unit": METRIC, "cores": threads,
            "kind": "reference" if kinds == {"reference"} else "port",
            "sample": "jobs %s of the mix (every %d-th), bands of rows in proportion to their pixels: %d pixel "
                      "paths, %.1f s%s" % (list(idx), idx[1] - idx[0] if len(idx) > 1 else 1, pix, t,
                                           "".join(sorted(notes))),
            "samples_per_s": pix / t if t > 0 else 0.0}


def run_reference(args, rank, ws, dist):
    if rank != 0:
        return
    scene = scene_for(args.config)
    from yune_gb300 import scenes
    seeds = scenes.pass_seeds(0, args.steps + args.warmup)
    cb = cpu_reference(scene, seeds, args.cpu_seconds, band=1 if args.config in ("c4", "c4_mis") else 0)
    cfg = {"workload": workload_string(args.config, scene), "spp_total": scene.spp,
           "reference_cfg": scene.cfg}
    line = {"metric": METRIC, "value": cb["value"], "unit": METRIC, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "fp32", "data": "synthetic", "config": cfg,
            "cpu_baseline": cb, "e2e": {"value": cb["value"], "unit": METRIC, "h2d_bytes_per_step": 0,
                                        "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def _reduce(dist, t_s, rays):
    """max of the ranks' times, sum of their rays (replicas)"""
    if not dist:
        return t_s, rays
    import torch
    mx = torch.tensor([t_s], dtype=torch.float64)
    dist.all_reduce(mx, op=dist.ReduceOp.MAX)
    sm = torch.tensor([float(rays)], dtype=torch.float64)
    dist.all_reduce(sm, op=dist.ReduceOp.SUM)
    return mx.item(), sm.item()


def replay_sample(jobs, seeds, every=128):
    """Algorithmic traversal work per walked ray, by kind: the rays an oracle pass walks a
    BVH with (the same rays the core walks) over every `every`-th row of each job's frame
    (so each job contributes in proportion to its pixels, as in the mix), replayed one at
    a time on the host in the device walk's order without the warp's speculation
    (yc_walk_counts). Returns {"closest"|"any": (rays, boxes, tris)}."""
    from oracle import oracle_py as O
    from yune_gb300 import scenes
    out = {"closest": [0, 0, 0], "any": [0, 0, 0]}
    for s, sd in zip(jobs, seeds):
        parts = [O.record_rays(s, int(sd[0]), s.cfg, (y, y + 1)) for y in range(every // 2, s.height, every)]
        rec = np.concatenate(parts) if parts else np.zeros((0, 8), np.float32)
        for name, sel in (("closest", rec[:, 7] < 2), ("any", rec[:, 7] >= 2)):
            r9 = O.rays9_of(rec[sel])
            if len(r9) == 0:
                continue
            b, t, _, _ = scenes.walk_counts(s, r9, any_hit=(name == "any"))
            out[name][0] += len(r9)
            out[name][1] += b
            out[name][2] += t
    return {k: tuple(v) for k, v in out.items()}


# DRAM bytes (read + write) per walked ray of k_batch_trace_mixed on the mixed workload
# with the default tree (mode 1) and the tuned shape (4 slot groups, traversal grid at
# 50%, 128-thread blocks): one ncu capture (dram__bytes_read.sum + dram__bytes_write.sum,
# one pass) of all 576 launches of two passes of the 64 jobs (`bench.py --traffic-only`
# with that shape under ncu), 85,934,615,808 + 7,993,981,696 bytes over 452,296,636
# walked rays. A launch's traffic is this figure times the rays it walks.
MIX_TRACE_DRAM_BYTES_PER_RAY = (85934615808 + 7993981696) / 452296636


def host_frames(sizes):
    """Page-locked (h, w, 4) float32 host buffers for the tonemapped frames the e2e steps
    read back, allocated before the timed region and reused step after step (plain numpy
    arrays where page-locked memory cannot be had)."""
    out = []
    for (w, h) in sizes:
        try:
            import torch
            out.append(torch.empty((h, w, 4), dtype=torch.float32, pin_memory=True).numpy())
        except Exception:
            out.append(np.empty((h, w, 4), np.float32))
    return out


def _trace_roofline(st, kt, l2, pk, pk_kind, kernel_mixed, kernel_extend, replay=None, dram_per_ray=None):
    """Roofline of the traversal kernel over its event time. achieved: the algorithmic
    bytes of the rays it walked -- 32 B per child box and 48 B per triangle a lone walk of
    the ray needs (replay: per-ray counts from the host replay of a sample of the same
    rays), plus 64 B of shading record fetched per closest-hit ray -- with the number of
    rays of each kind from the device counters. executed_*: the same with the boxes and
    triangles the device tested (its counters, speculation included) and 84 B of ray and
    hit records per ray. With the mixed kernel (both ray kinds in one launch) both kinds
    count; otherwise the closest-hit (extend) kernel alone."""
    mixed = kt.get("trace_launches", 0) > 0
    kinds = ("ext", "any") if mixed else ("ext",)
    boxes = sum(st[k + "_boxes"] for k in kinds)
    tris = sum(st[k + "_tris"] for k in kinds)
    rays = sum(st[k + "_rays"] for k in kinds)
    ms = kt["trace_ms"] if mixed else kt["extend_ms"]
    ex_bytes = 32.0 * boxes + 48.0 * tris + 84.0 * rays
    ex_achieved = ex_bytes / (ms / 1e3) / 1e9 if ms > 0 else 0.0
    if replay:
        alg = 0.0
        per_kind = {}
        for k, name, rec_b in (("ext", "closest", 64.0), ("any", "any", 0.0)):
            if k not in kinds:
                continue
            n, b, t = replay[name]
            per_ray = (32.0 * b + 48.0 * t) / n + rec_b if n else 0.0
            per_kind[name] = {"sample_rays": n, "boxes_per_ray": b / n if n else 0.0,
                              "tris_per_ray": t / n if n else 0.0, "bytes_per_ray": per_ray}
            alg += per_ray * st[k + "_rays"]
        nbytes, source = alg, "host replay of sampled rays (yc_walk_counts), no speculation"
    else:
        nbytes, source, per_kind = ex_bytes, "device counters (speculation included)", None
    achieved = nbytes / (ms / 1e3) / 1e9 if ms > 0 else 0.0
    out = {"kernel": kernel_mixed if mixed else kernel_extend, "bound": "l2", "achieved": achieved, "peak": l2,
           "unit": "GB/s", "frac": achieved / l2 if l2 else None, "traffic": None,
           "bytes_source": source, "replay": per_kind,
           "executed_achieved": ex_achieved, "executed_frac": ex_achieved / l2 if l2 else None,
           "executed_bytes_per_ray": ex_bytes / max(1, rays), "speculation_ratio": ex_bytes / nbytes if nbytes else None,
           "peak_source": "measured L2 read bandwidth (yc_measure_l2_gbs, 48 MB x 20 sweeps)",
           "hbm_peak": pk.get("hbm_gbs"), "hbm_frac": achieved / pk.get("hbm_gbs", 1.0), "hbm_peak_source": pk_kind,
           "rays": int(rays), "bytes_per_ray": nbytes / max(1, rays),
           # the device's tests in the reference's layouts (80 B BVHNodeGPU per box, 112 B
           # TriangleGPU per triangle, include/CL_headers.h:57-107)
           "ref_layout_bytes_per_ray": (80.0 * boxes + 112.0 * tris + 84.0 * rays) / max(1, rays),
           "ref_layout_achieved": ((80.0 * boxes + 112.0 * tris + 84.0 * rays) / (ms / 1e3) / 1e9 if ms > 0 else 0.0),
           "box_tests_per_ray": boxes / max(1, rays), "tri_tests_per_ray": tris / max(1, rays),
           "grays_per_s": rays / (ms / 1e3) / 1e9 if ms > 0 else 0.0}
    if mixed:
        out["closest_rays"] = int(st["ext_rays"])
        out["any_rays"] = int(st["any_rays"])
        launches = kt.get("trace_launches", 0)
        if dram_per_ray and launches:
            out["traffic"] = dram_per_ray * rays / launches
            out["traffic_source"] = ("DRAM bytes per walked ray from one ncu capture of this kernel on this "
                                     "workload, times the rays per launch of this run")
            out["algorithmic_bytes_per_launch"] = nbytes / launches
    return out


def run_ours(args, rank, local, ws, dist):
    """C1 on one GPU (a replica per rank under torchrun).

    A. per-pass drop-in path: W warm-up passes, then K timed passes, one yc_render_pass
       each (L2 flushed before each), per-kernel CUDA events;
    B. the whole job through the batch engine: the same frame, W warm-up passes as one
       job, then the K timed passes as one job (the value; path state of the pool is far
       larger than L2), and its image compared bit for bit with A's;
    C. a profiled copy of B without the graph (per-kernel events: split and roofline);
    D. e2e through the C-ABI with host buffers: per step the camera and the pass seeds go
       host -> device, the step's passes render, and the tonemapped frame comes back;
       once through the engine (E passes per step) and once per pass (yc_render_pass).
    """
    from yune_gb300 import autotune, quality, scenes
    from yune_gb300.batch import Batch
    from yune_gb300.core import Renderer
    scene = scene_for(args.config)
    K, Wm, E = args.steps, args.warmup, args.e2e_passes
    seeds = scenes.pass_seeds(0, Wm + 2 * K + args.e2e_steps * (E + 1))
    W, H = scene.width, scene.height
    r = Renderer(local)
    r.set_tree_mode(args.tree)
    r.set_tail_paths(args.tail)
    r.set_stack_smem(args.stack_smem)
    r.set_mixed_trace(args.mixed)
    r.set_ray_sort(args.ray_sort // 10, args.ray_sort % 10, args.ray_sort_min)
    r.set_shade_sort(args.shade_sort_min)
    sid = r.upload(scene)
    r.set_camera(scene.cam)
    l2 = r.measure_l2_gbs(48 << 20, 20)
    pk, pk_kind = peaks()

    # A. per pass
    aid = r.alloc_accum(W, H)
    for k in range(Wm):
        r.render(sid, aid, seeds[k], reset=1 if k == 0 else 0, cfg=scene.cfg)
    r.synchronize()
    r.reset_stats()
    r.set_profiling(True)
    pp_ms = 0.0
    for k in range(K):
        r.flush_l2(256 << 20)
        r.render(sid, aid, seeds[Wm + k], reset=0, cfg=scene.cfg)
        pp_ms += r.last_pass_ms()
    r.synchronize()
    st_pp = r.stats()
    kt_pp = r.kernel_times()
    r.set_profiling(False)
    img_pp = r.read_accum(aid)

    # B. the whole job through the engine, in the launch shape the autotuner picks for this
    #    frame (untimed calibration passes with seeds of their own), unless --pool fixes it
    cap = r.scene_depth(sid) + 2
    if args.pool:
        shape = dict(pool_paths=args.pool, rounds_per_launch=8, logic_blocks_per_sm=2, sort_threshold=1 << 16,
                     groups=args.groups, ray_sort=0)
        tune_info = None
    else:
        tuned, trials, tune_s = autotune.tune_scenes(r, [scene], [sid], stack_cap=cap)
        shape = tuned.kwargs()
        tune_info = {"seconds": tune_s, "trials": len(trials)}
    pool = shape["pool_paths"]
    aid_e = r.alloc_accum(W, H)
    b = Batch(r, stack_cap=cap, **shape)
    b.add_job(sid, aid_e, scene.cam, seeds[:Wm], scene.cfg, reset_first=1)
    b.run()
    b.add_job(sid, aid_e, scene.cam, seeds[Wm:Wm + K], scene.cfg, reset_first=0)
    r.flush_l2(256 << 20)
    r.synchronize()
    r.reset_stats()
    if dist:
        dist.barrier()
    with Clocks(local) as clk:
        b.run()
    en_ms = r.last_pass_ms()
    st_en = r.stats()
    img_en = r.read_accum(aid_e)
    same = bool(np.array_equal(img_en.view(np.int32), img_pp.view(np.int32)))
    b.close()

    # C. profiled copy of B (no graph): kernel split and the extend kernel's roofline
    aid_p = r.alloc_accum(W, H)
    bp = Batch(r, stack_cap=cap, use_graph=False, **shape)
    bp.add_job(sid, aid_p, scene.cam, seeds[Wm + K:Wm + 2 * K], scene.cfg, reset_first=1)
    r.flush_l2(256 << 20)
    r.reset_stats()
    r.set_profiling(True)
    bp.run()
    kt_en = r.kernel_times()
    st_enp = r.stats()
    r.set_profiling(False)
    bp.close()
    r.free_accum(aid_p)

    # D. e2e with host buffers
    base = Wm + 2 * K
    ldr = host_frames([(W, H)])[0]
    be = Batch(r, stack_cap=cap, **shape)
    r.reset_stats()
    t0 = time.perf_counter()
    for k in range(args.e2e_steps):
        be.add_job(sid, aid_e, scene.cam, seeds[base + k * E:base + (k + 1) * E], scene.cfg, reset_first=0)
        be.run()
        r.tonemap(aid_e, out=ldr)
    e2e_s = time.perf_counter() - t0
    e2e_rays = r.stats()["rays"]
    be.close()
    base += args.e2e_steps * E
    r.reset_stats()
    t0 = time.perf_counter()
    for k in range(args.e2e_steps):
        r.set_camera(scene.cam)
        r.render(sid, aid, seeds[base + k], reset=0, cfg=scene.cfg)
        r.tonemap(aid, out=ldr)
    e2e_pp_s = time.perf_counter() - t0
    e2e_pp_rays = r.stats()["rays"]

    t_s, rays = _reduce(dist, en_ms / 1e3, st_en["rays"])
    pp_s, pp_rays = _reduce(dist, pp_ms / 1e3, st_pp["rays"])
    e2e_s, e2e_rays = _reduce(dist, e2e_s, e2e_rays)
    e2e_pp_s, e2e_pp_rays = _reduce(dist, e2e_pp_s, e2e_pp_rays)
    if rank != 0:
        r.close()
        return
    launches = int(2 * kt_en["raygen_launches"] + kt_en["extend_launches"] + kt_en["occlusion_launches"]
                   + kt_en["trace_launches"] + kt_en["logic_launches"] + 3 * kt_en["sort_launches"]
                   + 2 * kt_en["raysort_launches"])   # engine: fill = plan + fill, ray sort = scan + scatter
    line = {
        "metric": METRIC, "value": rays / t_s / 1e6, "unit": METRIC, "n_gpus": ws, "steps": K,
        "warmup": Wm, "ms_per_step": en_ms / K, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32", "data": "synthetic (seeded procedural scene)",
        "config": {"workload": workload_string(args.config, scene),
                   "method": "the K steps rendered as one job of K passes through the batch engine",
                   "spp_total": scene.spp, "tree_mode": args.tree,
                   "l2": "L2 flushed before the timed job of K passes; its working set (path state of %d slots, "
                         "%d MB accumulator, %d MB scene) is %d MB, above the 126 MB L2"
                         % (pool, W * H * 16 >> 20, r.scene_bytes(sid) >> 20,
                            (pool * 232 + W * H * 16 + r.scene_bytes(sid)) >> 20),
                   "engine_shape": shape, "autotune": tune_info,
                   "parallelism": "replicas" if ws > 1 else "single GPU"},
        "samples_per_s": st_en["samples"] * (ws if dist else 1) / t_s,
        "rays_per_sample": st_en["rays"] / max(1, st_en["samples"]),
        "gpu_launches": launches,
        "engine_equal_to_per_pass": same,
        "kernel_ms": {"fill": kt_en["raygen_ms"], "raysort": kt_en["raysort_ms"], "trace": kt_en["trace_ms"],
                      "extend": kt_en["extend_ms"],
                      "occlusion": kt_en["occlusion_ms"], "sort": kt_en["sort_ms"], "logic": kt_en["logic_ms"],
                      "rounds": kt_en["rounds"]},
        "roofline": _trace_roofline(st_enp, kt_en, l2, pk, pk_kind, "k_batch_trace_mixed (closest + any-hit rays)",
                                    "k_batch_trace<closest> (extend)"),
        "per_pass": {"value": pp_rays / pp_s / 1e6, "ms_per_step": pp_ms / K, "unit": METRIC,
                     "note": "yc_render_pass per pass (the drop-in call), L2 flushed before each pass",
                     "kernel_ms": {"raygen": kt_pp["raygen_ms"], "raysort": kt_pp["raysort_ms"],
                                   "sort": kt_pp["sort_ms"], "trace": kt_pp["trace_ms"],
                                   "extend": kt_pp["extend_ms"], "occlusion": kt_pp["occlusion_ms"],
                                   "logic": kt_pp["logic_ms"], "tail": kt_pp["tail_ms"], "rounds": kt_pp["rounds"]},
                     "roofline": _trace_roofline(st_pp, kt_pp, l2, pk, pk_kind,
                                                 "k_trace_paths_mixed (closest + any-hit rays)",
                                                 "k_trace_paths<closest> (extend)")},
        "e2e": {"value": e2e_rays / e2e_s / 1e6 if e2e_s > 0 else 0.0, "unit": METRIC, "passes_per_step": E,
                "h2d_bytes_per_step": 80 + 4 * E, "d2h_bytes_per_step": W * H * 16, "steps": args.e2e_steps,
                "path": "yc_batch_add_job + yc_batch_run + yc_tonemap into a page-locked host buffer"},
        "e2e_per_pass": {"value": e2e_pp_rays / e2e_pp_s / 1e6 if e2e_pp_s > 0 else 0.0, "unit": METRIC,
                         "h2d_bytes_per_step": 80 + 4, "d2h_bytes_per_step": W * H * 16, "steps": args.e2e_steps,
                         "path": "yc_set_camera + yc_render_pass + yc_tonemap into a page-locked host buffer"},
        "clocks": clk.summary(),
        "image_error": quality.report(img_en, args.config, int(img_en[0, 0, 3])),
        "stack_overflow": int(st_en["stack_overflow"] + st_pp["stack_overflow"]),
        "image_mean": float(np.nanmean(img_en[..., :3])),
    }
    if not args.no_cpu:
        line["cpu_baseline"] = cpu_reference(scene, seeds, args.cpu_seconds)
    r.close()
    print(json.dumps(line))


WORKLOAD_NAMES = {
    "c0": "Cornell box (5 Oren-Nayar walls, seeded-yaw boxes, one Phong n=50), quad light",
    "c1": "glass icosphere (level 6, IOR 1.5) in the Cornell box",
    "c0_bdpt": "Cornell box, four quad lights, naive BDPT with 8 vertices per subpath",
    "c4": "stress: 40x40 grid of displaced level-4/5 icospheres, mixed materials, 4 quad lights, naive BDPT with "
          "8 vertices per subpath",
    "c0_mis": "Cornell box (5 Oren-Nayar walls, seeded-yaw boxes, one Phong n=50), quad light",
    "c0_bdpt_mis": "Cornell box, four quad lights",
    "c4_mis": "stress: 40x40 grid of displaced level-4/5 icospheres, mixed materials, 4 quad lights",
}


def workload_string(name, scene):
    """The workload a bench line is quoted on (the same string in both arms)."""
    W, H = scene.width, scene.height
    if scene.cfg.get("integrator", 0) == 2:
        return ("%s: %s, %d tris, %dx%d, %d lights, bidirectional path tracing with MIS (power heuristic), paths "
                "of at most %d segments, 1 spp per step"
                % (name, WORKLOAD_NAMES.get(name, name), scene.n_tri, W, H, len(scene.lights),
                   scene.cfg["bdpt_bounces"]))
    if scene.cfg.get("integrator", 0) == 1:
        return ("%s: %s, %d tris, %dx%d, %d lights, BDPT with %d vertices per subpath, 1 spp per step"
                % (name, WORKLOAD_NAMES.get(name, name), scene.n_tri, W, H, len(scene.lights),
                   scene.cfg["bdpt_bounces"]))
    return ("%s: %s, %d tris, %dx%d, 1 spp per step, NEE+MIS, RR after bounce %d, max depth %d"
            % (name, WORKLOAD_NAMES.get(name, name), scene.n_tri, W, H, scene.cfg["rr_threshold"],
               scene.cfg["max_depth"]))


def run_perpass_bdpt(args, rank, local, ws, dist):
    """BDPT configurations (c0_bdpt, and c4: 10M triangles, 3840x2160, naive BDPT with 8
    vertices per subpath and four lights) through yc_render_pass (the drop-in call), one
    pass per step. For c4 the node and triangle set (about 0.7 GB) is far larger than L2,
    so the traversal kernel's roofline is the HBM copy bandwidth."""
    from yune_gb300 import quality, scenes
    from yune_gb300.core import Renderer
    t0 = time.perf_counter()
    make = scenes.CONFIGS[args.config]
    if args.res:
        w, h = (int(x) for x in args.res.lower().split("x"))
        scene = make(width=w, height=h)
    else:
        scene = make()
    build_s = time.perf_counter() - t0
    K, Wm = args.steps, args.warmup
    seeds = scenes.pass_seeds(0, Wm + K + args.e2e_steps)
    W, H = scene.width, scene.height
    r = Renderer(local)
    r.set_tree_mode(args.tree)
    r.set_mixed_trace(args.mixed)
    r.set_stack_smem(args.stack_smem)
    r.set_ray_sort(args.ray_sort // 10, args.ray_sort % 10, args.ray_sort_min)
    r.set_shade_sort(args.shade_sort_min)
    t0 = time.perf_counter()
    sid = r.upload(scene)
    r.synchronize()
    upload_s = time.perf_counter() - t0
    scene_bytes = r.scene_bytes(sid)
    # the upload's repack on the host (YC_OPT_REPACK 0) against the device (the default),
    # each uploading a second copy of the scene: time and equal bytes
    repack = {}
    if args.tree == 1:
        digest = r.scene_digest(sid)
        for mode, key in ((0, "host_s"), (1, "device_s")):
            r.set_repack(mode)
            t0 = time.perf_counter()
            sid2 = r.upload(scene)
            r.synchronize()
            repack[key] = time.perf_counter() - t0
            repack["equal" if mode == 0 else "repeatable"] = r.scene_digest(sid2) == digest
            r.release(sid2)
        r.set_repack(1)
        repack["what"] = ("yc_upload_scene of the scene (checks, repack, copies) with the repack on the host "
                          "threads and on the device; equal: the host repack's arrays have the device repack's "
                          "digest; repeatable: a second device repack too")
    # the reference BVH of this scene built on the host (yh_bvh_build) and on the GPU
    # (yc_bvh_build), compared node for node
    leaf = 4 if args.config in ("c4", "c4_mis") else 10
    t0 = time.perf_counter()
    h_nodes, _ = scenes.build_bvh(scene.tris, 20, leaf)
    host_bvh_s = time.perf_counter() - t0
    r.build_bvh(scene.tris, 20, leaf)   # warm-up (allocation, module load)
    t0 = time.perf_counter()
    g_nodes, _ = r.build_bvh(scene.tris, 20, leaf)
    gpu_bvh_s = time.perf_counter() - t0
    bvh_equal = bool(len(g_nodes) == len(h_nodes) and all(np.array_equal(g_nodes[k], h_nodes[k]) for k in
                                                          ("p_min", "p_max", "child_idx", "vert_len")))
    del h_nodes, g_nodes
    r.set_camera(scene.cam)
    l2 = r.measure_l2_gbs(48 << 20, 20)
    pk, pk_kind = peaks()
    aid = r.alloc_accum(W, H)
    for k in range(Wm):
        r.render(sid, aid, seeds[k], reset=1 if k == 0 else 0, cfg=scene.cfg)
    r.synchronize()
    r.reset_stats()
    r.set_profiling(True)
    if dist:
        dist.barrier()
    ms = 0.0
    with Clocks(local) as clk:
        for k in range(K):
            r.flush_l2(256 << 20)
            r.render(sid, aid, seeds[Wm + k], reset=0, cfg=scene.cfg)
            ms += r.last_pass_ms()
    r.synchronize()
    st = r.stats()
    kt = r.kernel_times()
    r.set_profiling(False)
    # e2e through the C-ABI with host buffers: camera in, tonemapped frame out per step
    frame = host_frames([(W, H)])[0]
    r.reset_stats()
    t0 = time.perf_counter()
    for k in range(args.e2e_steps):
        r.set_camera(scene.cam)
        r.render(sid, aid, seeds[Wm + K + k], reset=0, cfg=scene.cfg)
        r.tonemap(aid, out=frame)
    e2e_s = time.perf_counter() - t0
    e2e_rays = r.stats()["rays"]
    img = r.read_accum(aid)
    t_s, rays = _reduce(dist, ms / 1e3, st["rays"])
    e2e_s, e2e_rays = _reduce(dist, e2e_s, e2e_rays)
    if rank != 0:
        r.close()
        return
    roof = _trace_roofline(st, kt, l2, pk, pk_kind, "k_trace_paths_mixed (closest + any-hit rays)",
                           "k_trace_paths<closest> (extend)")
    big = scene_bytes > L2_BYTES
    if big:   # the node and triangle set does not fit in L2: the bound is HBM
        roof.update({"bound": "hbm", "peak": pk.get("hbm_gbs"), "frac": roof["hbm_frac"], "peak_source": pk_kind,
                     "l2_peak": l2, "l2_frac": roof["achieved"] / l2 if l2 else None})
        for k in ("hbm_peak", "hbm_frac", "hbm_peak_source"):
            roof.pop(k, None)
    launches = int(kt["raygen_launches"] + kt["extend_launches"] + kt["occlusion_launches"] + kt["trace_launches"]
                   + kt["logic_launches"] + kt["tail_launches"] + 3 * kt["raysort_launches"] + 3 * kt["sort_launches"])
    line = {
        "metric": METRIC, "value": rays / t_s / 1e6, "unit": METRIC, "n_gpus": ws, "steps": K, "warmup": Wm,
        "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
        "data": "synthetic (seeded procedural scene)",
        "config": {"workload": workload_string(args.config, scene),
                   "spp_total": scene.spp, "tree_mode": args.tree, "scene_device_bytes": scene_bytes,
                   "host_build_s": build_s, "upload_s": upload_s, "repack": repack,
                   "bvh_build": {"host_s": host_bvh_s, "gpu_s": gpu_bvh_s, "equal": bvh_equal,
                                 "what": "BVH::createBVH node array, 20 bins, leaf <= %d: yh_bvh_build on the host "
                                         "core against yc_bvh_build on the GPU (host copy of the nodes included)"
                                         % leaf},
                   "l2": "L2 flushed before each step" + ("; the node and triangle set is larger than L2" if big else ""),
                   "parallelism": "replicas" if ws > 1 else "single GPU"},
        "samples_per_s": st["samples"] * (ws if dist else 1) / t_s,
        "rays_per_sample": st["rays"] / max(1, st["samples"]),
        "gpu_launches": launches,
        "kernel_ms": {"raygen": kt["raygen_ms"], "raysort": kt["raysort_ms"], "sort": kt["sort_ms"],
                      "trace": kt["trace_ms"], "extend": kt["extend_ms"],
                      "occlusion": kt["occlusion_ms"], "logic": kt["logic_ms"], "rounds": kt["rounds"]},
        "roofline": roof,
        "e2e": {"value": e2e_rays / e2e_s / 1e6 if e2e_s > 0 else 0.0, "unit": METRIC,
                "h2d_bytes_per_step": 80 + 4, "d2h_bytes_per_step": W * H * 16, "steps": args.e2e_steps,
                "path": "yc_set_camera + yc_render_pass + yc_tonemap into a page-locked host buffer"},
        "clocks": clk.summary(), "stack_overflow": int(st["stack_overflow"]),
        "image_mean": float(np.nanmean(img[..., :3])),
        "image_error": (quality.report(img, args.config, int(img[0, 0, 3]))
                        if quality.load_reference(args.config) is not None and not args.res else
                        "no FP64 reference for this scene (65,536 passes of the CPU oracle over 10M triangles "
                        "is out of reach); the BDPT integrator's error is measured on c0_bdpt"),
    }
    if not args.no_cpu:
        line["cpu_baseline"] = cpu_reference(scene, seeds, args.cpu_seconds, band=1 if big else 0)
    r.close()
    print(json.dumps(line))


# ---- the mixed workload (c2): batched against plain ----
def mix_cfg():
    """Render options of every job of the mix: NEE + MIS, Oren-Nayar diffuse, roulette
    after bounce 3, at most 16 bounces, the reference's MIS arithmetic (no lobe fix)."""
    from yune_gb300 import scenes
    return scenes.default_cfg(max_depth=16, mis_lobe_fix=0)


def mix_config(args, jobs_meta):
    """The `config` of both arms' lines (same workload, same options)."""
    tris, px = jobs_meta
    return {"workload": "c2: %d seeded scenes (Cornell box + displaced icospheres, %d triangles in all, 1k-500k "
                        "each), resolutions from {256^2, 512^2, 1280x720, 1920x1080} (%d pixels per pass), "
                        "materials from {Oren-Nayar, Phong exp 10-200, dielectric IOR 1.3-1.7}; NEE + MIS, "
                        "roulette after bounce 3, max depth 16; one step = one pass of every job"
                        % (args.jobs, tris, px),
            "jobs": args.jobs, "triangles": tris, "pixels_per_pass": px, "spp_config": 64,
            "reference_cfg": mix_cfg()}


def mix_totals(specs):
    """(triangles, pixels per pass) of the mix, from its job specifications."""
    from yune_gb300 import workloads
    return (int(sum(workloads.mixed_scene_tris(sp[0]) for sp in specs)), int(sum(sp[2] * sp[3] for sp in specs)))


def mix_sample(n_jobs, every):
    return list(range(0, n_jobs, max(1, every)))


def run_mix(args, rank, local, ws, dist):
    """The mixed workload on one GPU (a replica per rank under torchrun).

    Per repetition (--reps, median reported): the K passes of every job through the plain
    path (yc_render_passes, job after job) and through one batch (yc_batch_*), each timed
    with CUDA events on the context stream, both continuing the same accumulators from
    the same W warm-up passes; afterwards every accumulator of the batch equals the plain
    one bit for bit. Then a profiled copy of the batched form (no graph; per-kernel
    events: split and roofline), one profiled plain pass, e2e with host buffers, and the
    CPU baseline on a sample of the jobs."""
    from yune_gb300 import autotune, scenes, workloads
    from yune_gb300.batch import Batch
    from yune_gb300.core import Renderer
    K, Wm, R, E, S = args.steps, args.warmup, args.reps, args.e2e_passes, args.e2e_steps
    t0 = time.perf_counter()
    jobs = workloads.c2_jobs(n_jobs=args.jobs, spp=64, max_tris=args.max_tris, cfg=mix_cfg())
    build_s = time.perf_counter() - t0
    tris = int(sum(s.n_tri for s in jobs))
    px = int(sum(s.width * s.height for s in jobs))
    assert (tris, px) == mix_totals(workloads.c2_specs(args.jobs, max_tris=args.max_tris))
    n_seeds = Wm + R * K + 2 + S * E
    seeds = [scenes.pass_seeds(1000 + i, n_seeds) for i in range(len(jobs))]
    r = Renderer(local)
    r.set_tree_mode(args.tree)
    r.set_mixed_trace(args.mixed)
    r.set_ray_sort(args.ray_sort // 10, args.ray_sort % 10, args.ray_sort_min)
    r.set_shade_sort(args.shade_sort_min)
    r.set_tail_paths(args.tail)
    r.set_stack_smem(args.stack_smem)
    t0 = time.perf_counter()
    sids = [r.upload(s) for s in jobs]
    upload_s = time.perf_counter() - t0
    scene_bytes = sum(r.scene_bytes(sid) for sid in sids)
    cap = max(r.scene_depth(sid) for sid in sids) + 2
    l2 = r.measure_l2_gbs(48 << 20, 20)
    pk, pk_kind = peaks()
    if args.shape:
        shape, trials, tune_s = autotune.BatchShape(**json.loads(args.shape)), [], 0.0
    elif args.pool:
        shape, trials, tune_s = autotune.BatchShape(pool_paths=args.pool), [], 0.0
    else:   # launch shape from the autotuner (untimed calibration, seeds of its own)
        shape, trials, tune_s = autotune.tune_scenes(r, jobs, sids, stack_cap=cap)
    cfg = mix_cfg()
    if args.traffic_only:
        acc = [r.alloc_accum(s.width, s.height) for s in jobs]
        bt = Batch(r, stack_cap=cap, use_graph=False, max_jobs=len(jobs), **shape.kwargs())
        for s, sid, a, sd in zip(jobs, sids, acc, seeds):
            bt.add_job(sid, a, s.cam, sd[:2], cfg, reset_first=1)
        r.synchronize()
        r.reset_stats()
        r.set_profiling(True)
        bt.run()
        kt_t, st_t = r.kernel_times(), r.stats()
        r.set_profiling(False)
        bt.close()
        if rank == 0:
            print(json.dumps({"traffic_run": "two passes of every job, batch engine without a graph",
                              "jobs": len(jobs), "shape": shape.kwargs(),
                              "walked_rays": int(st_t["ext_rays"] + st_t["any_rays"]),
                              "trace_launches": int(kt_t["trace_launches"]), "trace_ms": kt_t["trace_ms"]}))
        r.close()
        return
    acc_p = [r.alloc_accum(s.width, s.height) for s in jobs]
    acc_b = [r.alloc_accum(s.width, s.height) for s in jobs]
    # warm-up: W passes of every job in each form
    for s, sid, a, sd in zip(jobs, sids, acc_p, seeds):
        r.set_camera(s.cam)
        r.render_passes(sid, a, sd[:Wm], reset_first=1, cfg=cfg)
    b = Batch(r, stack_cap=cap, max_jobs=len(jobs) * (R + S + 2), **shape.kwargs())
    for s, sid, a, sd in zip(jobs, sids, acc_b, seeds):
        b.add_job(sid, a, s.cam, sd[:Wm], cfg, reset_first=1)
    b.run()
    r.synchronize()
    reps = []
    if dist:
        dist.barrier()
    with Clocks(local) as clk:
        for k in range(R):
            sl = slice(Wm + k * K, Wm + (k + 1) * K)
            r.reset_stats()
            r.event(0)
            for s, sid, a, sd in zip(jobs, sids, acc_p, seeds):
                r.set_camera(s.cam)
                r.render_passes(sid, a, sd[sl], reset_first=0, cfg=cfg)
            r.event(1)
            ms_p = r.elapsed_ms(0, 1)
            st_p = r.stats()
            for s, sid, a, sd in zip(jobs, sids, acc_b, seeds):
                b.add_job(sid, a, s.cam, sd[sl], cfg, reset_first=0)
            r.synchronize()
            r.reset_stats()
            r.event(2)
            left = b.run()
            r.event(3)
            ms_b = r.elapsed_ms(2, 3)
            st_b = r.stats()
            reps.append({"plain_ms": ms_p, "batched_ms": ms_b, "plain_rays": int(st_p["rays"]),
                         "batched_rays": int(st_b["rays"]), "batched_traversed": int(st_b["traversed"]),
                         "batched_samples": int(st_b["samples"]), "plain_samples": int(st_p["samples"]),
                         "unfinished": left, "overflow": int(st_p["stack_overflow"] + st_b["stack_overflow"])})
    same = True
    for a, c in zip(acc_p, acc_b):
        same = same and bool(np.array_equal(r.read_accum(a).view(np.int32), r.read_accum(c).view(np.int32)))
    # image error of the jobs with a converged FP64 reference (tests/golden/fp64_c2_j*.npz)
    from yune_gb300 import quality
    image_error = {}
    for j in (0, 8, 16):
        if j < len(jobs):
            rep_j = quality.report(r.read_accum(acc_b[j]), "c2_j%d" % j, Wm + R * K)
            if rep_j:
                image_error["c2_j%d" % j] = rep_j
    # profiled copies (per-kernel events; no graph): two passes of every job batched, one plain
    prof = slice(Wm + R * K, Wm + R * K + 2)
    scratch = [r.alloc_accum(s.width, s.height) for s in jobs]
    bp = Batch(r, stack_cap=cap, use_graph=False, max_jobs=len(jobs), **shape.kwargs())
    for s, sid, a, sd in zip(jobs, sids, scratch, seeds):
        bp.add_job(sid, a, s.cam, sd[prof], cfg, reset_first=1)
    r.synchronize()
    r.reset_stats()
    r.set_profiling(True)
    bp.run()
    kt_b = r.kernel_times()
    st_bp = r.stats()
    r.set_profiling(False)
    bp.close()
    # the same two passes with one slot group and the whole of each SM for the traversal:
    # the kernel's speed when no other group's kernels share its SMs
    alone = dict(shape.kwargs(), groups=1, trace_share=100)
    kt_a = st_a = None
    if (shape.groups, shape.trace_share) != (1, 100):
        ba = Batch(r, stack_cap=cap, use_graph=False, max_jobs=len(jobs), **alone)
        for s, sid, a, sd in zip(jobs, sids, scratch, seeds):
            ba.add_job(sid, a, s.cam, sd[prof], cfg, reset_first=1)
        r.synchronize()
        r.reset_stats()
        r.set_profiling(True)
        ba.run()
        kt_a, st_a = r.kernel_times(), r.stats()
        r.set_profiling(False)
        ba.close()
    r.reset_stats()
    r.set_profiling(True)
    for s, sid, a, sd in zip(jobs, sids, scratch, seeds):
        r.set_camera(s.cam)
        r.render_passes(sid, a, sd[prof][:1], reset_first=1, cfg=cfg)
    kt_p = r.kernel_times()
    st_pp = r.stats()
    r.set_profiling(False)
    for a in scratch:
        r.free_accum(a)
    # e2e through the C-ABI with host buffers: S steps of E passes of every job
    base = Wm + R * K + 2
    frames = host_frames([(s.width, s.height) for s in jobs])
    r.reset_stats()
    t0 = time.perf_counter()
    for k in range(S):
        for s, sid, a, sd in zip(jobs, sids, acc_b, seeds):
            b.add_job(sid, a, s.cam, sd[base + k * E:base + (k + 1) * E], cfg, reset_first=0)
        b.run()
        for a, f in zip(acc_b, frames):
            r.tonemap(a, out=f)
    e2e_s = time.perf_counter() - t0
    e2e_rays = r.stats()["rays"]
    r.reset_stats()
    t0 = time.perf_counter()
    for k in range(S):
        for s, sid, a, sd, f in zip(jobs, sids, acc_p, seeds, frames):
            r.set_camera(s.cam)
            r.render_passes(sid, a, sd[base + k * E:base + (k + 1) * E], reset_first=0, cfg=cfg)
            r.tonemap(a, out=f)
    e2e_p_s = time.perf_counter() - t0
    e2e_p_rays = r.stats()["rays"]
    b.close()
    idx = mix_sample(len(jobs), args.sample_every)
    t0 = time.perf_counter()
    replay = replay_sample([jobs[i] for i in idx], [seeds[i][prof.start:] for i in idx])
    replay_s = time.perf_counter() - t0
    med = lambda v: float(np.median(v))  # noqa: E731
    vb = [x["batched_rays"] / (x["batched_ms"] / 1e3) / 1e6 for x in reps]
    vp = [x["plain_rays"] / (x["plain_ms"] / 1e3) / 1e6 for x in reps]
    mid = int(np.argsort(vb)[len(vb) // 2])
    t_s, rays = _reduce(dist, reps[mid]["batched_ms"] / 1e3, reps[mid]["batched_rays"])
    e2e_s, e2e_rays = _reduce(dist, e2e_s, e2e_rays)
    e2e_p_s, e2e_p_rays = _reduce(dist, e2e_p_s, e2e_p_rays)
    if rank != 0:
        r.close()
        return
    # the profiled run's launches per pass, times K: the engine's fill is two kernels (plan,
    # fill), its ray sort two (scan, scatter: the keys come from the logic and fill kernels)
    launches = int(2 * kt_b["raygen_launches"] + kt_b["extend_launches"] + kt_b["occlusion_launches"]
                   + kt_b["trace_launches"] + kt_b["logic_launches"] + 3 * kt_b["sort_launches"]
                   + 2 * kt_b["raysort_launches"]) * K // 2
    acc_bytes = 16 * px
    line = {
        "metric": METRIC, "value": rays / t_s / 1e6, "unit": METRIC, "n_gpus": ws, "steps": K, "warmup": Wm,
        "ms_per_step": reps[mid]["batched_ms"] / K, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32", "data": "synthetic (seeded procedural scenes)",
        "config": dict(mix_config(args, (tris, px)),
                       method="the K steps of every job rendered as one batch of K passes per job (value), and job "
                              "after job through yc_render_passes (plain); median of %d repetitions" % R,
                       l2="inputs larger than L2: %d MB of scenes and %d MB of accumulators per form"
                          % (scene_bytes >> 20, acc_bytes >> 20),
                       engine_shape=shape.kwargs(), tree_mode=args.tree,
                       parallelism="replicas" if ws > 1 else "single GPU"),
        "batched_over_plain": med([a / b for a, b in zip(vb, vp)]),
        "plain": {"value": med(vp), "ms_per_step": med([x["plain_ms"] for x in reps]) / K, "unit": METRIC,
                  "samples_per_s": med([x["plain_samples"] / (x["plain_ms"] / 1e3) for x in reps]),
                  "path": "yc_set_camera + yc_render_passes, one call of K passes per job, job after job"},
        "reps": [dict(x, batched_mrays=a, plain_mrays=p) for x, a, p in zip(reps, vb, vp)],
        "equal_results": same,
        "samples_per_s": reps[mid]["batched_samples"] / (reps[mid]["batched_ms"] / 1e3),
        "walked_grays_per_s": reps[mid]["batched_traversed"] / (reps[mid]["batched_ms"] / 1e3) / 1e9,
        "rays_per_sample": reps[mid]["batched_rays"] / max(1, reps[mid]["batched_samples"]),
        "walked_share": reps[mid]["batched_traversed"] / max(1, reps[mid]["batched_rays"]),
        "gpu_launches": launches,
        "kernel_ms_2_passes": {"fill": kt_b["raygen_ms"], "raysort": kt_b["raysort_ms"], "trace": kt_b["trace_ms"],
                               "sort": kt_b["sort_ms"], "logic": kt_b["logic_ms"], "rounds": kt_b["rounds"]},
        "plain_kernel_ms_1_pass": {"raygen": kt_p["raygen_ms"], "raysort": kt_p["raysort_ms"],
                                   "trace": kt_p["trace_ms"], "sort": kt_p["sort_ms"], "logic": kt_p["logic_ms"],
                                   "tail": kt_p["tail_ms"], "rounds": kt_p["rounds"]},
        "roofline": _trace_roofline(st_bp, kt_b, l2, pk, pk_kind, "k_batch_trace_mixed (closest + any-hit rays)",
                                    "k_batch_trace<closest> (extend)", replay,
                                    dram_per_ray=MIX_TRACE_DRAM_BYTES_PER_RAY if args.tree == 1 else None),
        "plain_roofline": _trace_roofline(st_pp, kt_p, l2, pk, pk_kind, "k_trace_paths_mixed (closest + any-hit rays)",
                                          "k_trace_paths<closest> (extend)", replay),
        "e2e": {"value": e2e_rays / e2e_s / 1e6 if e2e_s > 0 else 0.0, "unit": METRIC, "passes_per_step": E,
                "steps": S, "h2d_bytes_per_step": len(jobs) * (80 + 4 * E), "d2h_bytes_per_step": acc_bytes,
                "path": "per step: yc_batch_add_job (camera, seeds) for every job + yc_batch_run + yc_tonemap of "
                        "every job into its page-locked host buffer"},
        "e2e_plain": {"value": e2e_p_rays / e2e_p_s / 1e6 if e2e_p_s > 0 else 0.0, "unit": METRIC,
                      "passes_per_step": E, "steps": S, "h2d_bytes_per_step": len(jobs) * (80 + 4 * E),
                      "d2h_bytes_per_step": acc_bytes,
                      "path": "per step and job: yc_set_camera + yc_render_passes + yc_tonemap into the job's page-locked host buffer"},
        "clocks": clk.summary(),
        "image_error": image_error,
        "host": {"scene_build_s": build_s, "upload_s": upload_s, "autotune_s": tune_s, "autotune_trials": len(trials),
                 "replay_s": replay_s},
        "stack_overflow": int(sum(x["overflow"] for x in reps)),
    }
    if kt_a is not None:
        # with several slot groups and a traversal grid below the whole SM, a traversal
        # launch shares the SMs with the other groups' kernels (and traversals), so its
        # event time -- the denominator of roofline.achieved -- counts that shared time
        line["roofline"]["concurrency"] = (
            "%d slot groups, traversal grid at %d%% of each SM's resident blocks: launches of the groups overlap, "
            "so the launch times count time shared with other kernels; roofline_alone is the kernel with the SMs "
            "to itself" % (shape.groups, shape.trace_share))
        line["roofline_alone"] = _trace_roofline(st_a, kt_a, l2, pk, pk_kind,
                                                 "k_batch_trace_mixed (closest + any-hit rays), one slot group, "
                                                 "whole SM", "k_batch_trace<closest> (extend)", replay,
                                                 dram_per_ray=MIX_TRACE_DRAM_BYTES_PER_RAY if args.tree == 1 else None)
        line["kernel_ms_2_passes_alone"] = {"trace": kt_a["trace_ms"], "logic": kt_a["logic_ms"],
                                            "sort": kt_a["sort_ms"], "raysort": kt_a["raysort_ms"]}
    if not args.no_cpu:
        line["cpu_baseline"] = cpu_reference_mix([jobs[i] for i in idx], idx, [seeds[i] for i in idx],
                                                 args.cpu_seconds)
    r.close()
    print(json.dumps(line))


def run_reference_mix(args, rank, ws, dist):
    """The reference arm on the mix: the compiled reference on the sampled jobs, whose
    scenes come from the oracle library's producers and whose BVHs come from the
    reference's BVH::createBVH -- no product library is loaded."""
    if rank != 0:
        return
    from oracle import oracle_py as O
    from yune_gb300 import scenes, workloads
    idx = mix_sample(args.jobs, args.sample_every)
    specs = workloads.c2_specs(args.jobs, max_tris=args.max_tris)
    with scenes.producers(O.scene_lib(), O.ref_bvh_with_depth):
        jobs = workloads.c2_jobs(n_jobs=args.jobs, spp=64, max_tris=args.max_tris, cfg=mix_cfg(), only=idx)
    n_seeds = args.warmup + args.reps * args.steps
    seeds = [scenes.pass_seeds(1000 + i, n_seeds) for i in idx]
    cb = cpu_reference_mix(jobs, idx, seeds, args.cpu_seconds)
    cfg = mix_config(args, mix_totals(specs))
    line = {"metric": METRIC, "value": cb["value"], "unit": METRIC, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "fp32", "data": "synthetic (seeded procedural scenes)", "config": cfg,
            "cpu_baseline": cb, "e2e": {"value": cb["value"], "unit": METRIC, "h2d_bytes_per_step": 0,
                                        "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_c3(args):
    """Served requests (continuous batching) against the plain first-come loop, for each
    arrival rate of --rates (or --rate), over the same resident scenes."""
    from yune_gb300 import autotune, scenes, serve, workloads
    from yune_gb300.core import Renderer
    t0 = time.perf_counter()
    resident = workloads.c3_scenes(8, max_tris=args.max_tris)
    build_s = time.perf_counter() - t0
    rates = [float(x) for x in args.rates.split(",")] if args.rates else [args.rate]
    r = Renderer(0)
    r.set_tree_mode(args.tree)
    r.set_mixed_trace(args.mixed)
    r.set_ray_sort(args.ray_sort // 10, args.ray_sort % 10, args.ray_sort_min)
    r.set_shade_sort(args.shade_sort_min)
    sids = [r.upload(s) for s in resident]
    cap = max(r.scene_depth(sid) for sid in sids) + 2
    if args.pool:
        shape, tune_s = autotune.BatchShape(pool_paths=args.pool), 0.0
    else:   # the server's launch shape from the tuner: every resident scene at 1024x1024
        t0 = time.perf_counter()
        sizes = [(1024, 1024)] * len(resident)
        n = autotune.calibration_passes(sum(w * h for w, h in sizes))
        cal = [(sid, s.cam, scenes.pass_seeds(4242 + i, n), s.cfg) for i, (s, sid) in enumerate(zip(resident, sids))]
        shape, _ = autotune.tune(r, cal, sizes, stack_cap=cap)
        tune_s = time.perf_counter() - t0
    srv = serve.Server(r, resident, hbm_budget=args.hbm_budget_mb << 20, shape=shape, sids=sids)
    runs = []
    for rate in rates:
        reqs = workloads.c3_requests(args.requests, rate, len(resident), res_range=(256, args.res_max),
                                     spp_range=(16, args.spp_max))
        mk = lambda: [serve.Request(a, sc, w, h, spp, seed=i) for i, (a, sc, w, h, spp) in enumerate(reqs)]  # noqa
        r.reset_stats()
        t0 = time.perf_counter()
        served = srv.run(mk())
        ts = time.perf_counter() - t0
        sts = r.stats()
        r.reset_stats()
        t0 = time.perf_counter()
        plain = serve.serve_plain(r, resident, mk())
        tpl = time.perf_counter() - t0
        stp = r.stats()
        p50s, p99s = serve.percentiles(served)
        p50p, p99p = serve.percentiles(plain)
        runs.append({"rate_per_s": rate, "requests": len(reqs),
                     "pixel_passes": int(sum(w * h * spp for (_, _, w, h, spp) in reqs)),
                     "served": {"p50": p50s, "p99": p99s, "Mrays_s": sts["rays"] / ts / 1e6, "seconds": ts,
                                "max_in_flight": srv.max_in_flight, "max_bytes_in_use": srv.max_in_use},
                     "plain": {"p50": p50p, "p99": p99p, "Mrays_s": stp["rays"] / tpl / 1e6, "seconds": tpl},
                     "rays_equal": sts["rays"] == stp["rays"]})
        srv.max_in_flight = srv.max_in_use = 0
    srv.close()
    out = {"metric": "p50/p99 time to target spp (s) and aggregate Mrays/s", "unit": "s",
           "config": {"workload": "c3 serving", "resolution": [256, args.res_max], "spp": [16, args.spp_max],
                      "scene_triangles": [int(s.n_tri) for s in resident], "hbm_budget_mb": args.hbm_budget_mb,
                      "engine_shape": shape.kwargs(), "autotune_s": tune_s, "host_build_s": build_s},
           "runs": runs}
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


def scenes_is_bdpt(name):
    return name in ("c0_bdpt", "c4", "c0_mis", "c0_bdpt_mis", "c4_mis")


def main():
    args = parse()
    if args.quality:
        return run_quality(args)
    if args.trace_bench:
        return run_trace_bench(args)
    if args.impl == "ours" and args.config == "c3":
        return run_c3(args)
    rank, local, ws, dist = dist_init(args)
    if args.impl == "reference":
        if args.config == "c2":
            run_reference_mix(args, rank, ws, dist)
        else:
            run_reference(args, rank, ws, dist)
    elif args.config == "c2":
        run_mix(args, rank, local, ws, dist)
    elif scenes_is_bdpt(args.config):
        run_perpass_bdpt(args, rank, local, ws, dist)
    else:
        run_ours(args, rank, local, ws, dist)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
