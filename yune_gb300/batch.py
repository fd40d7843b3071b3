"""Batch and serving front end over the engine of include/yune_cuda.h (yc_batch_*).

A Batch renders many jobs (scene, camera, accumulator, pass seeds) in one persistent
wavefront; every pixel's passes run in order, so a job's accumulator is bit-identical to
rendering it alone pass by pass with yc_render_pass.
"""
import ctypes as C

import numpy as np

from . import _native as N
from .core import cfg_struct
from .layouts import ptr


class Batch:
    def __init__(self, renderer, pool_paths=0, rounds_per_launch=0, logic_blocks_per_sm=0, use_graph=True,
                 max_jobs=0, stack_cap=0, sort_threshold=0, groups=0, ray_sort=0, trace_block=0, stack_smem=0,
                 trace_share=0):
        self.r = renderer
        self.L = renderer.L
        cfg = N.BatchCfg(pool_paths, rounds_per_launch, logic_blocks_per_sm, int(use_graph), max_jobs, stack_cap,
                         sort_threshold, groups, ray_sort, trace_block, stack_smem, trace_share)
        h = C.c_void_p()
        N.check(self.L.yc_batch_create(renderer.h, C.byref(cfg), C.byref(h)), "yc_batch_create")
        self.h = h
        self.jobs = []
        renderer._children.add(self)

    def add_job(self, scene_id, accum_id, cam, seeds, cfg, reset_first=1):
        s = np.ascontiguousarray(seeds, dtype=np.uint32)
        c = cfg_struct(cfg)
        jid = C.c_int()
        N.check(self.L.yc_batch_add_job(self.h, scene_id, accum_id, ptr(cam), ptr(s), len(s), reset_first,
                                        C.byref(c), C.byref(jid)), "yc_batch_add_job")
        self.jobs.append(jid.value)
        return jid.value

    def run(self, max_launches=0):
        """Runs up to max_launches graph launches (0: to completion); returns unfinished jobs."""
        left = C.c_int()
        N.check(self.L.yc_batch_run(self.h, max_launches, C.byref(left)), "yc_batch_run")
        return left.value

    def progress(self, job_id):
        d, t = C.c_int64(), C.c_int64()
        N.check(self.L.yc_batch_job_progress(self.h, job_id, C.byref(d), C.byref(t)), "yc_batch_job_progress")
        return d.value, t.value

    def cancel(self, job_id):
        """Stops a job between runs (yc_batch_cancel_job): its pixels in flight finish their
        current pass, the rest are counted done; progress reaches the total once its work
        in flight drains, and its accumulator must stay allocated until then."""
        N.check(self.L.yc_batch_cancel_job(self.h, job_id), "yc_batch_cancel_job")

    def close(self):
        if getattr(self, "h", None) and getattr(self.r, "h", None):
            self.L.yc_batch_destroy(self.h)
        self.h = None

    def _detach(self):
        # the renderer's context is being destroyed and releases this batch with it
        self.h = None

    def __del__(self):
        self.close()
