"""Render server: continuous batching of render requests over resident scenes.

A Python driver of the server in the C-ABI (yc_serve_*, core/serve.cpp): requests (scene,
resolution, target spp) arrive over time; a request is admitted when its accumulator fits
the HBM budget left by the requests in flight; it then becomes a job of one long-lived
batch, whose slots interleave the wavefronts of every admitted request and take new work
as pixels finish, so requests that arrive while others run start as soon as memory frees
up. Scenes stay resident; accumulators are freed when their request completes. Latency
is arrival to completion of the target spp (the spp is the RMSE target: the estimate is
the same at equal spp in any mix).

Failure handling, all on the host (the admission rules of yc_admission): a request whose
accumulator exceeds the whole budget is rejected, as is one that arrives while
`max_queue` requests already wait for memory; a request may carry a cancellation time
(seconds after its arrival): still waiting, it is dropped; admitted, its job is cancelled
in the engine (its pixels stop after their current pass) and its accumulator is freed
once that work drains. Each request ends with status "done", "rejected: ..." or
"cancelled".
"""
import ctypes as C
import time
from dataclasses import dataclass, field

import numpy as np

from . import _native as N
from . import scenes
from .core import cfg_struct


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
    job: int = -1                # the server's request id once submitted
    accum: int = -1              # the accumulator while admitted (-1 once freed or never)
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


STATUS = {N.REQ_DONE: "done", N.REQ_CANCELLED: "cancelled",
          N.REQ_REJECTED_BUDGET: "rejected: larger than the whole HBM budget",
          N.REQ_REJECTED_QUEUE: "rejected: queue full"}


class Server:
    def __init__(self, renderer, resident, hbm_budget, pool_paths=1 << 21, rounds_per_launch=8, keep_results=False,
                 cfg=None, logic_blocks_per_sm=2, sort_threshold=1 << 16, max_queue=None, scene_budget=None,
                 shape=None, sids=None):
        """scene_budget: device bytes the resident scenes may take together (None: no
        limit); checked on the host before anything is uploaded, as CLManager checks each
        buffer against the device's global memory before creating it
        (src/CLManager.cpp:428-429, 452-453). shape: an autotune.BatchShape for the
        server's batch (its fields replace pool_paths, rounds_per_launch,
        logic_blocks_per_sm and sort_threshold). sids: the resident scenes' ids when
        they are uploaded already (else they are uploaded here)."""
        self.r = renderer
        self.scenes = resident
        self.scene_bytes = None
        if scene_budget is not None:
            mode = getattr(renderer, "tree_mode", 1)   # the layout the uploads below will build
            self.scene_bytes = sum(scenes.device_bytes(s, tree_mode=mode) for s in resident)
            if self.scene_bytes > scene_budget:
                raise ValueError("resident scenes need %d device bytes, above the scene budget of %d"
                                 % (self.scene_bytes, scene_budget))
        self.sids = list(sids) if sids is not None else [renderer.upload(s) for s in resident]
        self.budget = int(hbm_budget)
        self.keep = keep_results
        self.cfg = cfg or scenes.default_cfg(max_depth=16)
        cap = max(renderer.scene_depth(sid) for sid in self.sids) + 2
        if shape is not None:
            bc = N.BatchCfg(shape.pool_paths, shape.rounds_per_launch, shape.logic_blocks_per_sm, 1, 1 << 16, cap,
                            shape.sort_threshold, shape.groups, shape.ray_sort, shape.trace_block, shape.stack_smem,
                            shape.trace_share)
        else:
            bc = N.BatchCfg(pool_paths, rounds_per_launch, logic_blocks_per_sm, 1, 1 << 16, cap, sort_threshold, 0, 0)
        sc = N.ServeCfg(self.budget, -1 if max_queue is None else int(max_queue), int(bool(keep_results)), bc)
        h = C.c_void_p()
        self.L = renderer.L
        N.check(self.L.yc_serve_create(renderer.h, C.byref(sc), C.byref(h)), "yc_serve_create")
        self.h = h
        self.max_queue = max_queue
        self.in_use = 0          # accumulator bytes of the requests in flight
        self.max_in_flight = 0   # most requests admitted at once, and most accumulator bytes
        self.max_in_use = 0

    def info(self, q):
        i = N.RequestInfo()
        N.check(self.L.yc_serve_info(self.h, q.job, C.byref(i)), "yc_serve_info")
        return i

    def _submit(self, q):
        s = self.scenes[q.scene]
        seeds = scenes.pass_seeds(q.seed, q.spp)
        d = N.RequestDesc()
        d.scene_id = self.sids[q.scene]
        d.width, d.height, d.n_pass = q.width, q.height, q.spp
        d.seeds_host = seeds.ctypes.data
        C.memmove(C.byref(d.cam), s.cam.ctypes.data, C.sizeof(N.Cam))
        d.cfg = cfg_struct(self.cfg)
        rid, st = C.c_int64(), C.c_int32()
        N.check(self.L.yc_serve_submit(self.h, C.byref(d), C.byref(rid), C.byref(st)), "yc_serve_submit")
        q.job = rid.value
        return st.value

    def run(self, requests, clock=time.perf_counter):
        """Serves the requests in real time; returns them (sorted by arrival) with their
        status and completion time."""
        pending = sorted(requests, key=lambda q: q.arrival)
        open_ = []   # submitted, not finished
        t0 = clock()
        i = 0
        running, waiting = C.c_int32(), C.c_int32()
        while i < len(pending) or open_:
            now = clock() - t0
            while i < len(pending) and pending[i].arrival <= now:
                q = pending[i]
                st = self._submit(q)
                if st in (N.REQ_REJECTED_BUDGET, N.REQ_REJECTED_QUEUE):
                    q.status, q.done = STATUS[st], now
                else:
                    q.status = "waiting" if st == N.REQ_WAITING else "running"
                    open_.append(q)
                i += 1
            for q in open_:
                if q.status in ("waiting", "running") and q.cancelled_by(now):
                    N.check(self.L.yc_serve_cancel(self.h, q.job), "yc_serve_cancel")
                    q.status = "cancelling"
            has_work = any(q.status in ("running", "cancelling", "waiting") for q in open_)
            N.check(self.L.yc_serve_step(self.h, 1 if has_work else 0, C.byref(running), C.byref(waiting)),
                    "yc_serve_step")
            now = clock() - t0
            still, in_use = [], 0
            for q in open_:
                inf = self.info(q)
                if inf.admit_s >= 0 and q.admitted < 0:
                    q.admitted = now
                if inf.state in (N.REQ_RUNNING, N.REQ_CANCELLING):
                    q.accum = inf.accum_id
                    in_use += q.bytes
                if inf.state in (N.REQ_DONE, N.REQ_CANCELLED):
                    q.done, q.status = now, STATUS[inf.state]
                    if inf.state == N.REQ_DONE and self.keep:
                        q.result = np.zeros((q.height, q.width, 4), np.float32)
                        N.check(self.L.yc_serve_read(self.h, q.job, q.result.ctypes.data), "yc_serve_read")
                        N.check(self.L.yc_serve_release(self.h, q.job), "yc_serve_release")
                else:
                    if inf.state == N.REQ_RUNNING and q.status == "waiting":
                        q.status = "running"
                    still.append(q)
            open_ = still
            self.in_use = in_use
            self.max_in_use = max(self.max_in_use, in_use)
            self.max_in_flight = max(self.max_in_flight, running.value)
            if not open_ and i < len(pending):
                time.sleep(max(0.0, pending[i].arrival - (clock() - t0)))
        return pending

    def close(self):
        if getattr(self, "h", None):
            self.L.yc_serve_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()


class Admission:
    """The admission rules alone (yc_admission_*), on the host: no device needed."""

    def __init__(self, budget, max_queue=None):
        h = C.c_void_p()
        L = N.lib()
        N.check(L.yc_admission_create(int(budget), -1 if max_queue is None else int(max_queue), C.byref(h)),
                "yc_admission_create")
        self.L, self.h = L, h

    def submit(self, nbytes):
        t, st = C.c_int64(), C.c_int32()
        N.check(self.L.yc_admission_submit(self.h, int(nbytes), C.byref(t), C.byref(st)), "yc_admission_submit")
        return t.value, st.value

    def next(self):
        t = C.c_int64()
        N.check(self.L.yc_admission_next(self.h, C.byref(t)), "yc_admission_next")
        return t.value

    def cancel(self, t):
        st = C.c_int32()
        N.check(self.L.yc_admission_cancel(self.h, int(t), C.byref(st)), "yc_admission_cancel")
        return st.value

    def finish(self, t):
        st = C.c_int32()
        N.check(self.L.yc_admission_finish(self.h, int(t), C.byref(st)), "yc_admission_finish")
        return st.value

    def state(self, t):
        st = C.c_int32()
        N.check(self.L.yc_admission_state(self.h, int(t), C.byref(st)), "yc_admission_state")
        return st.value

    def usage(self):
        b, w, r = C.c_uint64(), C.c_int32(), C.c_int32()
        N.check(self.L.yc_admission_usage(self.h, C.byref(b), C.byref(w), C.byref(r)), "yc_admission_usage")
        return b.value, w.value, r.value

    def close(self):
        if getattr(self, "h", None):
            self.L.yc_admission_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()


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
