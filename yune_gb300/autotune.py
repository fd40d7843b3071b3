"""Autotuner for the batch engine's launch shape.

The batch engine (yc_batch_*) has six free parameters that change speed but never
results: the number of path slots in flight (the wavefront size), the rounds captured
in one CUDA graph launch, the logic kernel's blocks per SM, the queue size from which
the shade queue is sorted by path phase and material class (0: never), the number of
slot groups whose rounds run concurrently, and whether each round's rays are sorted by
origin and direction cell before the trace. The best values depend
on the job mix (total pixels, scene sizes, path lengths), so the tuner times candidate
shapes on a calibration run of the mix itself: every job's first passes, into scratch
accumulators, with the engine's own CUDA-event clock (yc_last_pass_ms); small mixes
render several passes per job so that the calibration sees the steady state. It
searches one parameter at a time (pool size, rounds per launch, logic blocks, sort threshold,
groups, ray sort) from a measured starting shape, keeping the best value of each before
moving on, and sweeps once more if the first sweep changed the shape.
"""
import time
from dataclasses import dataclass

from . import scenes
from .batch import Batch

POOLS = (1 << 19, 1 << 20, 1 << 21, 1 << 22)
ROUNDS = (4, 8, 16)
LOGIC_BLOCKS = (2, 4, 8)
SORT = (0, 1 << 16, 1 << 18)
GROUPS = (1, 2, 4)
RAY_SORT = (-1, 32)   # rays in queue order, or sorted by 3 origin and 2 direction bits per axis


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

    def kwargs(self):
        return dict(pool_paths=self.pool_paths, rounds_per_launch=self.rounds_per_launch,
                    logic_blocks_per_sm=self.logic_blocks_per_sm, sort_threshold=self.sort_threshold,
                    groups=self.groups, ray_sort=self.ray_sort)


def calibration_passes(total_px):
    """Passes per job of a calibration run: enough pixel passes to fill the largest pool
    four times over, so that slots regenerate and the wavefront reaches its steady mix
    of path phases (one pass of a frame no larger than the pool is a single wave of
    fresh paths, which favours other shapes than a long job does); at most 16."""
    return max(1, min(16, -(-4 * POOLS[-1] // max(1, total_px))))


def _calibrate(renderer, jobs, shape, stack_cap, accs, passes=1):
    """Milliseconds of `passes` passes of every job under `shape` (device time of
    yc_batch_run)."""
    b = Batch(renderer, stack_cap=stack_cap, **shape.kwargs())
    try:
        for (sid, cam, seeds, cfg), a in zip(jobs, accs):
            b.add_job(sid, a, cam, seeds[:passes], cfg)
        b.run()
        return renderer.last_pass_ms()
    finally:
        b.close()


def tune(renderer, jobs, sizes, stack_cap=0, log=None):
    """Picks a BatchShape for `jobs`, a list of (scene_id, cam, seeds, cfg) tuples, whose
    frames have the (width, height) of `sizes`. Returns (shape, trials) where trials lists
    (shape, ms) in the order they were timed."""
    accs = [renderer.alloc_accum(w, h) for (w, h) in sizes]
    total_px = sum(w * h for (w, h) in sizes)
    passes = min(calibration_passes(total_px), min(len(j[2]) for j in jobs))
    trials = []
    try:
        best = BatchShape()
        best.pool_paths = min(best.pool_paths, _round_pool(total_px))
        best_ms = _calibrate(renderer, jobs, best, stack_cap, accs, passes)
        trials.append((BatchShape(**best.kwargs()), best_ms))
        timed = {tuple(sorted(best.kwargs().items())): best_ms}
        for sweep in range(2):   # a second sweep only when the first one moved
            start = BatchShape(**best.kwargs())
            for field, values in (("pool_paths", POOLS), ("rounds_per_launch", ROUNDS),
                                  ("logic_blocks_per_sm", LOGIC_BLOCKS), ("sort_threshold", SORT),
                                  ("groups", GROUPS), ("ray_sort", RAY_SORT)):
                for v in values:
                    if v == getattr(best, field):
                        continue
                    if field == "pool_paths" and v > _round_pool(total_px):
                        continue   # more slots than pixels stay idle
                    cand = BatchShape(**best.kwargs())
                    setattr(cand, field, v)
                    key = tuple(sorted(cand.kwargs().items()))
                    if key in timed:
                        continue
                    ms = _calibrate(renderer, jobs, cand, stack_cap, accs, passes)
                    timed[key] = ms
                    trials.append((cand, ms))
                    if log:
                        log("autotune %s -> %.2f ms" % (cand, ms))
                    if ms < best_ms:
                        best, best_ms = cand, ms
            if best == start:
                break
    finally:
        for a in accs:
            renderer.free_accum(a)
    return best, trials


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
