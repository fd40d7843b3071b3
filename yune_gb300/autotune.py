"""Autotuner for the batch engine's launch shape: a Python front end of yc_batch_tune
(core/tune.cpp, in the C-ABI so that a C or C++ host tunes the same way).

The batch engine (yc_batch_*) has nine free parameters that change speed but never
results: the number of path slots in flight (the wavefront size), the rounds captured in
one CUDA graph launch, the logic kernel's blocks per SM, the queue size from which the
shade queue is sorted by path phase and material class (0: never), the number of slot
groups whose rounds run concurrently, whether each round's rays are sorted by origin and
direction cell before the trace, the traversal kernels' block shape (threads per
block: with the per-thread stack columns it sets the shared memory per block, hence the
blocks and the L1 left per SM), how many entries of each walk's stack stay in shared
memory (the deeper ones spill to global memory; fewer leave more L1), and the share of
each SM the persistent traversal grid takes (below 100% the other slot groups' kernels
run beside it; searched together with the number of groups). The best values depend on the job mix (total pixels,
scene sizes, path lengths), so the tuner times candidate shapes on a calibration run of
the mix itself: every job's first passes, into scratch accumulators, with the engine's own
CUDA-event clock; small mixes render several passes per job so that the calibration sees
the steady state. It searches one parameter at a time from a measured starting shape,
keeping the best value of each before moving on, and sweeps once more if the first sweep
changed the shape. The traversal stack depth is what the deepest scene needs.
"""
import ctypes as C
import time
from dataclasses import dataclass

import numpy as np

from . import _native as N
from . import scenes
from .core import cfg_struct

POOLS = (1 << 19, 1 << 20, 1 << 21, 1 << 22)


@dataclass
class BatchShape:
    """A launch shape; the defaults are the search's starting point (the best shape
    measured by hand on the glass-sphere frame and the mixed batch)."""
    pool_paths: int = 1 << 21
    rounds_per_launch: int = 8
    logic_blocks_per_sm: int = 2
    sort_threshold: int = 1 << 16
    groups: int = 2
    ray_sort: int = 0
    trace_block: int = 128
    stack_smem: int = 12
    trace_share: int = 100

    def kwargs(self):
        return dict(pool_paths=self.pool_paths, rounds_per_launch=self.rounds_per_launch,
                    logic_blocks_per_sm=self.logic_blocks_per_sm, sort_threshold=self.sort_threshold,
                    groups=self.groups, ray_sort=self.ray_sort, trace_block=self.trace_block,
                    stack_smem=self.stack_smem, trace_share=self.trace_share)

    @staticmethod
    def of(cfg):
        return BatchShape(cfg.pool_paths, cfg.rounds_per_launch, cfg.logic_blocks_per_sm, cfg.sort_threshold,
                          cfg.groups, cfg.ray_sort, cfg.trace_block, cfg.stack_smem, cfg.trace_share)

    def cfg(self, stack_cap=0, use_graph=1):
        """The yc_batch_cfg of this shape."""
        return N.BatchCfg(self.pool_paths, self.rounds_per_launch, self.logic_blocks_per_sm, use_graph, 0, stack_cap,
                          self.sort_threshold, self.groups, self.ray_sort, self.trace_block, self.stack_smem,
                          self.trace_share)


def calibration_passes(total_px):
    """Passes per job of a calibration run: enough pixel passes to fill the largest pool
    four times over, so that slots regenerate and the wavefront reaches its steady mix
    of path phases (one pass of a frame no larger than the pool is a single wave of
    fresh paths, which favours other shapes than a long job does); at most 16."""
    return max(1, min(16, -(-4 * POOLS[-1] // max(1, total_px))))


def tune(renderer, jobs, sizes, stack_cap=0, log=None, sweeps=2):
    """Picks a BatchShape for `jobs`, a list of (scene_id, cam, seeds, cfg) tuples, whose
    frames have the (width, height) of `sizes`, with yc_batch_tune. Returns (shape,
    trials) where trials lists (shape, ms) in the order they were timed."""
    total_px = sum(w * h for (w, h) in sizes)
    passes = min(calibration_passes(total_px), min(len(j[2]) for j in jobs))
    arr = (N.TuneJob * len(jobs))()
    keep = []
    for t, (sid, cam, seeds, cfg), (w, h) in zip(arr, jobs, sizes):
        sd = np.ascontiguousarray(seeds[:passes], np.uint32)
        keep.append(sd)
        C.memmove(C.byref(t.cam), np.ascontiguousarray(cam).ctypes.data, C.sizeof(N.Cam))
        t.cfg = cfg_struct(cfg)
        t.scene_id, t.width, t.height, t.n_pass, t.seeds_host = sid, w, h, passes, sd.ctypes.data
    start = BatchShape().cfg(stack_cap)
    cap = 256
    out = N.BatchCfg()
    tr = (N.TuneTrial * cap)()
    n = C.c_int()
    N.check(renderer.L.yc_batch_tune(renderer.h, arr, len(jobs), C.byref(start), sweeps, C.byref(out), tr, cap,
                                     C.byref(n)), "yc_batch_tune")
    trials = [(BatchShape.of(tr[i].cfg), float(tr[i].ms)) for i in range(min(n.value, cap))]
    if log:
        for sh, ms in trials:
            log("autotune %s -> %.2f ms" % (sh, ms))
    return BatchShape.of(out), trials


def search(start, total_px, clock, sweeps=2):
    """The tuner's search alone (yc_tune_search) over clock(shape) -> time: no device.
    Returns (best shape, [(shape, time)] in the order timed)."""
    def cb(cfg, _user):
        return float(clock(BatchShape.of(cfg.contents)))
    fn = N.TUNE_CLOCK(cb)
    st = start.cfg()
    out = N.BatchCfg()
    cap = 256
    tr = (N.TuneTrial * cap)()
    n = C.c_int()
    N.check(N.lib().yc_tune_search(C.byref(st), int(total_px), sweeps, C.cast(fn, C.c_void_p), None, C.byref(out), tr,
                                   cap, C.byref(n)), "yc_tune_search")
    return BatchShape.of(out), [(BatchShape.of(tr[i].cfg), float(tr[i].ms)) for i in range(min(n.value, cap))]


def _round_pool(total_px):
    p = 1 << 16
    while p < total_px and p < POOLS[-1]:
        p <<= 1
    return p


def tune_scenes(renderer, scene_list, sids, seed=4242, stack_cap=0, log=None):
    """tune() for SceneData records already uploaded as `sids` (calibration seeds are
    drawn independently of the seeds the jobs render with)."""
    sizes = [(s.width, s.height) for s in scene_list]
    n = calibration_passes(sum(w * h for (w, h) in sizes))
    jobs = [(sid, s.cam, scenes.pass_seeds(seed + i, n), s.cfg) for i, (s, sid) in enumerate(zip(scene_list, sids))]
    t0 = time.perf_counter()
    shape, trials = tune(renderer, jobs, sizes, stack_cap=stack_cap, log=log)
    return shape, trials, time.perf_counter() - t0
