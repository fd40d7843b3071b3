"""Serving: requests admitted while others run, each result equal to rendering it alone."""
import numpy as np
import pytest

from yune_gb300 import scenes, serve
from yune_gb300.core import Renderer

pytestmark = pytest.mark.gpu


def test_served_results_equal_alone_and_budget_respected():
    resident = [scenes.c0(8, 8), scenes.c1(8, 8, level=3)]
    reqs = [serve.Request(0.0, 0, 32, 24, 3, seed=1), serve.Request(0.0, 1, 20, 20, 2, seed=2),
            serve.Request(0.01, 0, 16, 40, 4, seed=3), serve.Request(0.02, 1, 40, 16, 2, seed=4)]
    with Renderer(0) as r:
        # budget for about two accumulators at a time: later requests wait for memory
        srv = serve.Server(r, resident, hbm_budget=2 * 32 * 24 * 16 + 64, pool_paths=700, rounds_per_launch=2,
                           keep_results=True)
        done = srv.run(reqs)
        srv.close()
        assert all(q.done >= q.arrival for q in done)
        sids = [r.upload(s) for s in resident]
        for q in done:
            s = resident[q.scene]
            r.set_camera(s.cam)
            aid = r.alloc_accum(q.width, q.height)
            r.render_passes(sids[q.scene], aid, scenes.pass_seeds(q.seed, q.spp), reset_first=1,
                            cfg=scenes.default_cfg(max_depth=16))
            alone = r.read_accum(aid)
            assert np.array_equal(q.result.view(np.int32), alone.view(np.int32))
        p50, p99 = serve.percentiles(done)
        assert 0 <= p50 <= p99


def test_cancelled_and_rejected_requests():
    """A request cancelled while it runs stops in the engine and frees its accumulator; one
    cancelled while it waits never reaches the engine; one larger than the budget is
    rejected; the others still equal their lone renders."""
    resident = [scenes.c0(8, 8)]
    reqs = [serve.Request(0.0, 0, 64, 64, 16384, seed=1, cancel_after=0.05),
            serve.Request(0.0, 0, 64, 64, 2, seed=2, cancel_after=0.01),
            serve.Request(0.0, 0, 32, 32, 2, seed=3),
            serve.Request(0.0, 0, 128, 128, 2, seed=4)]
    with Renderer(0) as r:
        srv = serve.Server(r, resident, hbm_budget=reqs[0].bytes + 64, pool_paths=1024, rounds_per_launch=2,
                           keep_results=True)
        done = srv.run(reqs)
        srv.close()
        st = [q.status for q in done]
        assert st == ["cancelled", "cancelled", "done", "rejected: larger than the whole HBM budget"]
        assert done[1].job == -1 and srv.in_use == 0
        q = done[2]
        sid = r.upload(resident[0])
        r.set_camera(resident[0].cam)
        aid = r.alloc_accum(q.width, q.height)
        r.render_passes(sid, aid, scenes.pass_seeds(q.seed, q.spp), reset_first=1,
                        cfg=scenes.default_cfg(max_depth=16))
        assert np.array_equal(q.result.view(np.int32), r.read_accum(aid).view(np.int32))
