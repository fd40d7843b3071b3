"""The batch engine against the per-pass path: jobs of different scenes, resolutions and
pass counts rendered together must give, per job, exactly the accumulator the per-pass
path gives alone (each pixel's passes run in order in one slot)."""
import ctypes as C

import numpy as np
import pytest

from yune_gb300 import scenes
from yune_gb300.batch import Batch
from yune_gb300.core import Renderer

pytestmark = pytest.mark.gpu


def _jobs():
    a = scenes.c0(40, 30)
    b = scenes.c1(24, 36, level=4)
    c = scenes.c0(17, 9, seed=5)
    return [(a, scenes.pass_seeds(1, 3)), (b, scenes.pass_seeds(2, 2)), (c, scenes.pass_seeds(3, 5))]


# stack_smem: walk-stack entries in shared memory (0: the default 12; 1, 2, 4: most of
# each walk's stack in the global spill area; 64: all of it in shared memory); share: the
# traversal grid's percent of the resident blocks (0: 100; 10: one block per SM)
@pytest.mark.parametrize("use_graph,pool,sort,groups,tb,smem,share",
                         [(True, 4096, 0, 1, 0, 0, 0), (False, 1000, 0, 2, 64, 4, 50),
                          (True, 1 << 16, 0, 2, 256, 2, 0), (True, 4096, 1, 3, 32, 64, 25),
                          (False, 1000, 64, 4, 128, 1, 10), (True, 999, 0, 8, 96, 12, 75)])
def test_batch_matches_per_pass(use_graph, pool, sort, groups, tb, smem, share):
    jobs = _jobs()
    with Renderer(0) as r:
        ids = []
        for s, seeds in jobs:
            sid = r.upload(s)
            ids.append(sid)
        want = []
        for (s, seeds), sid in zip(jobs, ids):
            r.set_camera(s.cam)
            aid = r.alloc_accum(s.width, s.height)
            r.render_passes(sid, aid, seeds, reset_first=1, cfg=s.cfg)
            want.append(r.read_accum(aid))
        b = Batch(r, pool_paths=pool, rounds_per_launch=4, use_graph=use_graph, sort_threshold=sort, groups=groups,
                  trace_block=tb, stack_smem=smem, trace_share=share)
        accs = []
        for (s, seeds), sid in zip(jobs, ids):
            aid = r.alloc_accum(s.width, s.height)
            accs.append(aid)
            b.add_job(sid, aid, s.cam, seeds, s.cfg)
        assert b.run() == 0
        for (s, _), aid, w, jid in zip(jobs, accs, want, b.jobs):
            got = r.read_accum(aid)
            assert np.array_equal(got.view(np.int32), w.view(np.int32))
            assert b.progress(jid) == (s.width * s.height, s.width * s.height)
        b.close()


@pytest.mark.parametrize("groups,smem", [(1, 0), (2, 2)])
def test_batch_separate_trace_launches_match(groups, smem):
    """With one traversal launch per ray kind (YC_OPT_MIXED_TRACE = 0) the batch gives the
    same accumulators as the per-pass path, as with the mixed launch."""
    jobs = _jobs()
    with Renderer(0) as r:
        r.set_mixed_trace(0)
        ids = [r.upload(s) for s, _ in jobs]
        want = []
        for (s, seeds), sid in zip(jobs, ids):
            r.set_camera(s.cam)
            aid = r.alloc_accum(s.width, s.height)
            r.render_passes(sid, aid, seeds, reset_first=1, cfg=s.cfg)
            want.append(r.read_accum(aid))
        b = Batch(r, pool_paths=4096, rounds_per_launch=4, use_graph=True, groups=groups, stack_smem=smem)
        accs = []
        for (s, seeds), sid in zip(jobs, ids):
            aid = r.alloc_accum(s.width, s.height)
            accs.append(aid)
            b.add_job(sid, aid, s.cam, seeds, s.cfg)
        assert b.run() == 0
        for aid, w in zip(accs, want):
            assert np.array_equal(r.read_accum(aid).view(np.int32), w.view(np.int32))
        b.close()


@pytest.mark.parametrize("groups,key", [(1, 0), (3, 0), (2, 322), (1, 111)])
def test_batch_ray_sort_matches(groups, key):
    """With every round's rays sorted by origin and direction cell (threshold 1), or by
    job and cell (key = job bits * 100 + origin bits * 10 + direction bits), the batch
    still gives the per-pass path's accumulators bit for bit."""
    jobs = _jobs()
    with Renderer(0) as r:
        ids = [r.upload(s) for s, _ in jobs]
        want = []
        for (s, seeds), sid in zip(jobs, ids):
            r.set_camera(s.cam)
            aid = r.alloc_accum(s.width, s.height)
            r.render_passes(sid, aid, seeds, reset_first=1, cfg=s.cfg)
            want.append(r.read_accum(aid))
        r.set_ray_sort(3, 2, min_rays=1)
        b = Batch(r, pool_paths=4096, rounds_per_launch=4, use_graph=True, groups=groups, ray_sort=key)
        accs = []
        for (s, seeds), sid in zip(jobs, ids):
            aid = r.alloc_accum(s.width, s.height)
            accs.append(aid)
            b.add_job(sid, aid, s.cam, seeds, s.cfg)
        assert b.run() == 0
        for aid, w in zip(accs, want):
            assert np.array_equal(r.read_accum(aid).view(np.int32), w.view(np.int32))
        b.close()


def test_batch_jobs_added_while_running():
    """Serving: a job admitted after the batch started still renders exactly."""
    jobs = _jobs()
    with Renderer(0) as r:
        sids = [r.upload(s) for s, _ in jobs]
        cap = max(r.scene_depth(sid) for sid in sids) + 2   # the stack is fixed once the batch runs
        b = Batch(r, pool_paths=512, rounds_per_launch=2, stack_cap=cap)
        a0 = r.alloc_accum(jobs[0][0].width, jobs[0][0].height)
        b.add_job(sids[0], a0, jobs[0][0].cam, jobs[0][1], jobs[0][0].cfg)
        b.run(max_launches=3)
        a1 = r.alloc_accum(jobs[1][0].width, jobs[1][0].height)
        b.add_job(sids[1], a1, jobs[1][0].cam, jobs[1][1], jobs[1][0].cfg)
        assert b.run() == 0
        got1 = r.read_accum(a1)
        r.set_camera(jobs[1][0].cam)
        a_ref = r.alloc_accum(jobs[1][0].width, jobs[1][0].height)
        r.render_passes(sids[1], a_ref, jobs[1][1], reset_first=1, cfg=jobs[1][0].cfg)
        assert np.array_equal(got1.view(np.int32), r.read_accum(a_ref).view(np.int32))
        b.close()


def test_autotuned_shape_gives_identical_results():
    """The tuner only picks a launch shape: the tuned batch renders the same bits."""
    from yune_gb300 import autotune
    jobs = _jobs()
    with Renderer(0) as r:
        sids = [r.upload(s) for s, _ in jobs]
        cap = max(r.scene_depth(sid) for sid in sids) + 2
        shape, trials, _ = autotune.tune_scenes(r, [s for s, _ in jobs], sids, stack_cap=cap)
        assert trials and all(ms > 0 for _, ms in trials)
        assert shape.pool_paths >= 1 << 16
        b = Batch(r, stack_cap=cap, **shape.kwargs())
        accs = []
        for (s, seeds), sid in zip(jobs, sids):
            accs.append(r.alloc_accum(s.width, s.height))
            b.add_job(sid, accs[-1], s.cam, seeds, s.cfg)
        assert b.run() == 0
        for (s, seeds), sid, aid in zip(jobs, sids, accs):
            r.set_camera(s.cam)
            ref = r.alloc_accum(s.width, s.height)
            r.render_passes(sid, ref, seeds, reset_first=1, cfg=s.cfg)
            assert np.array_equal(r.read_accum(aid).view(np.int32), r.read_accum(ref).view(np.int32))
        b.close()


@pytest.mark.parametrize("groups", [1, 2])
def test_cancelled_job_drains_and_others_are_unchanged(groups):
    """yc_batch_cancel_job between runs: the cancelled job's pixels stop after their
    current pass (fewer passes than asked, none more) and the job drains to done; the
    other job, and a job added after the cancellation, give exactly their per-pass
    accumulators."""
    a = scenes.c0(48, 40)
    b = scenes.c1(24, 36, level=4)
    with Renderer(0) as r:
        sa, sb = r.upload(a), r.upload(b)
        want = []
        for s, sid, seeds in ((b, sb, scenes.pass_seeds(2, 6)), (a, sa, scenes.pass_seeds(3, 2))):
            r.set_camera(s.cam)
            aid = r.alloc_accum(s.width, s.height)
            r.render_passes(sid, aid, seeds, reset_first=1, cfg=s.cfg)
            want.append(r.read_accum(aid))
        bt = Batch(r, pool_paths=600, rounds_per_launch=2, groups=groups)
        acc_a = r.alloc_accum(a.width, a.height)
        acc_b = r.alloc_accum(b.width, b.height)
        ja = bt.add_job(sa, acc_a, a.cam, scenes.pass_seeds(1, 64), a.cfg)
        jb = bt.add_job(sb, acc_b, b.cam, scenes.pass_seeds(2, 6), b.cfg)
        bt.run(max_launches=1)
        bt.cancel(ja)
        acc_c = r.alloc_accum(a.width, a.height)
        jc = bt.add_job(sa, acc_c, a.cam, scenes.pass_seeds(3, 2), a.cfg)
        assert bt.run() == 0
        n = a.width * a.height
        assert bt.progress(ja) == (n, n)
        passes = r.read_accum(acc_a)[..., 3]
        assert passes.max() < 64 and passes.min() >= 0
        assert np.array_equal(r.read_accum(acc_b).view(np.int32), want[0].view(np.int32))
        assert np.array_equal(r.read_accum(acc_c).view(np.int32), want[1].view(np.int32))
        assert bt.progress(jc) == (n, n) and bt.progress(jb) == (b.width * b.height,) * 2
        bt.close()


@pytest.mark.parametrize("field,value", [("trace_share", 5), ("trace_share", 101), ("trace_block", 48),
                                         ("groups", 9), ("stack_smem", -1)])
def test_batch_refuses_bad_shapes(field, value):
    """yc_batch_create refuses a launch shape outside its ranges with YC_E_INVALID."""
    from yune_gb300 import _native as N
    with Renderer(0) as r:
        cfg = N.BatchCfg(4096, 4, 2, 1, 0, 0, 0, 0, 0, 0, 0, 0)
        setattr(cfg, field, value)
        h = C.c_void_p()
        assert r.L.yc_batch_create(r.h, C.byref(cfg), C.byref(h)) == N.YC_E_INVALID
