"""Render server: continuous batching of render requests over resident scenes.

Requests (scene, resolution, target spp) arrive over time. A request is admitted when
its accumulator fits the HBM budget left by the requests in flight; it then becomes a
job of one long-lived batch (yune_gb300.batch), whose slots interleave the wavefronts of
every admitted request and take new work as pixels finish, so requests that arrive
while others run start as soon as memory frees up. Scenes stay resident; accumulators
are freed when their request completes. Latency is arrival to completion of the target
spp (the spp is the RMSE target: the estimate is the same at equal spp in any mix).

Failure handling, all on the host: a request whose accumulator exceeds the whole budget
is rejected, as is one that arrives while `max_queue` requests already wait for memory;
a request may carry a cancellation time (seconds after its arrival): still waiting, it is
dropped; admitted, its job is cancelled in the engine (yc_batch_cancel_job: its pixels
stop after their current pass) and its accumulator is freed once that work drains. Each
request ends with status "done", "rejected: ..." or "cancelled".
"""
import time
from dataclasses import dataclass, field

import numpy as np

from . import scenes
from .batch import Batch


@dataclass
class Request:
    arrival: float
    scene: int
    width: int
    height: int
    spp: int
    seed: int = 0
    cancel_after: float = None   # seconds after arrival at which the client cancels
    # filled in by the server
    admitted: float = -1.0
    done: float = -1.0
    job: int = -1
    accum: int = -1
    status: str = "pending"
    result: np.ndarray = field(default=None, repr=False)

    @property
    def bytes(self):
        return self.width * self.height * 16 + self.spp * 4

    @property
    def latency(self):
        return self.done - self.arrival

    def cancelled_by(self, now):
        return self.cancel_after is not None and now >= self.arrival + self.cancel_after


class Server:
    def __init__(self, renderer, resident, hbm_budget, pool_paths=1 << 21, rounds_per_launch=8, keep_results=False,
                 cfg=None, logic_blocks_per_sm=2, sort_threshold=1 << 16, max_queue=None, scene_budget=None):
        """scene_budget: device bytes the resident scenes may take together (None: no
        limit); checked on the host before anything is uploaded, as CLManager checks each
        buffer against the device's global memory before creating it
        (src/CLManager.cpp:428-429, 452-453)."""
        self.r = renderer
        self.scenes = resident
        self.scene_bytes = None
        if scene_budget is not None:
            mode = getattr(renderer, "tree_mode", 1)   # the layout the uploads below will build
            self.scene_bytes = sum(scenes.device_bytes(s, tree_mode=mode) for s in resident)
            if self.scene_bytes > scene_budget:
                raise ValueError("resident scenes need %d device bytes, above the scene budget of %d"
                                 % (self.scene_bytes, scene_budget))
        self.sids = [renderer.upload(s) for s in resident]
        self.budget = int(hbm_budget)
        self.in_use = 0
        self.keep = keep_results
        self.cfg = cfg or scenes.default_cfg(max_depth=16)
        cap = max(renderer.scene_depth(sid) for sid in self.sids) + 2
        self.batch = Batch(renderer, pool_paths=pool_paths, rounds_per_launch=rounds_per_launch, max_jobs=4096,
                           stack_cap=cap, logic_blocks_per_sm=logic_blocks_per_sm, sort_threshold=sort_threshold)
        self.max_queue = max_queue   # requests waiting for memory beyond this are rejected
        self.max_in_flight = 0   # most requests admitted at once, and most accumulator bytes
        self.max_in_use = 0

    def _admit(self, q, now):
        if self.in_use + q.bytes > self.budget:
            return False
        s = self.scenes[q.scene]
        q.accum = self.r.alloc_accum(q.width, q.height)
        q.job = self.batch.add_job(self.sids[q.scene], q.accum, s.cam, scenes.pass_seeds(q.seed, q.spp), self.cfg)
        q.admitted = now
        self.in_use += q.bytes
        self.max_in_use = max(self.max_in_use, self.in_use)
        return True

    def _arrive(self, q, waiting, live, now):
        if q.bytes > self.budget:
            q.status, q.done = "rejected: larger than the whole HBM budget", now
        elif not waiting and self._admit(q, now):
            q.status = "running"
            live.append(q)
        elif self.max_queue is not None and len(waiting) >= self.max_queue:
            q.status, q.done = "rejected: queue full", now
        else:
            waiting.append(q)

    def run(self, requests, clock=time.perf_counter):
        """Serves the requests in real time; returns them (sorted by arrival) with their
        status and completion time."""
        pending = sorted(requests, key=lambda q: q.arrival)
        waiting, live = [], []
        t0 = clock()
        i = 0
        while i < len(pending) or waiting or live:
            now = clock() - t0
            while i < len(pending) and pending[i].arrival <= now:
                self._arrive(pending[i], waiting, live, now)
                i += 1
            # cancellations: waiting requests are dropped, admitted ones stop in the engine
            for q in [q for q in waiting if q.cancelled_by(now)]:
                waiting.remove(q)
                q.status, q.done = "cancelled", now
            for q in live:
                if q.status == "running" and q.cancelled_by(now):
                    self.batch.cancel(q.job)
                    q.status = "cancelling"
            # admission in arrival order while memory allows
            while waiting and self._admit(waiting[0], now):
                q = waiting.pop(0)
                q.status = "running"
                live.append(q)
            self.max_in_flight = max(self.max_in_flight, len(live))
            if not live:   # (a waiting request always fits an empty budget)
                if i < len(pending):
                    time.sleep(max(0.0, pending[i].arrival - (clock() - t0)))
                continue
            self.batch.run(max_launches=1)
            now = clock() - t0
            still = []
            for q in live:
                d, tot = self.batch.progress(q.job)
                if d >= tot:
                    q.done = now
                    if q.status == "cancelling":
                        q.status = "cancelled"
                    else:
                        q.status = "done"
                        if self.keep:
                            q.result = self.r.read_accum(q.accum)
                    self.r.free_accum(q.accum)
                    self.in_use -= q.bytes
                else:
                    still.append(q)
            live = still
        return pending

    def close(self):
        self.batch.close()


def serve_plain(renderer, resident, requests, cfg=None, clock=time.perf_counter, keep_results=False):
    """The plain loop: requests one at a time, first come first served, each rendered
    pass by pass with yc_render_pass (the reference's per-frame dispatch)."""
    cfg = cfg or scenes.default_cfg(max_depth=16)
    sids = [renderer.upload(s) for s in resident]
    pending = sorted(requests, key=lambda q: q.arrival)
    t0 = clock()
    for q in pending:
        now = clock() - t0
        if q.arrival > now:
            time.sleep(q.arrival - now)
        q.admitted = clock() - t0
        s = resident[q.scene]
        renderer.set_camera(s.cam)
        aid = renderer.alloc_accum(q.width, q.height)
        renderer.render_passes(sids[q.scene], aid, scenes.pass_seeds(q.seed, q.spp), reset_first=1, cfg=cfg)
        renderer.synchronize()
        q.done = clock() - t0
        if keep_results:
            q.result = renderer.read_accum(aid)
        renderer.free_accum(aid)
    return pending


def percentiles(reqs):
    """p50 and p99 latency of the completed requests."""
    lat = np.array([q.latency for q in reqs if q.status in ("pending", "done")])
    return float(np.percentile(lat, 50)), float(np.percentile(lat, 99))
