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
        assert done[1].accum == -1 and srv.in_use == 0     # the waiting one never held an accumulator
        q = done[2]
        sid = r.upload(resident[0])
        r.set_camera(resident[0].cam)
        aid = r.alloc_accum(q.width, q.height)
        r.render_passes(sid, aid, scenes.pass_seeds(q.seed, q.spp), reset_first=1,
                        cfg=scenes.default_cfg(max_depth=16))
        assert np.array_equal(q.result.view(np.int32), r.read_accum(aid).view(np.int32))


def test_server_starts_within_its_scene_budget():
    resident = [scenes.c0(8, 8), scenes.c1(8, 8, level=3)]
    need = sum(scenes.device_bytes(s) for s in resident)
    with Renderer(0) as r:
        srv = serve.Server(r, resident, hbm_budget=1 << 20, scene_budget=need, pool_paths=1024)
        assert srv.scene_bytes == need == sum(r.scene_bytes(sid) for sid in srv.sids)
        srv.close()


def test_serve_c_abi_directly():
    """yc_serve_* driven as a C host would: submit, step until done, read, release; the
    result equals the lone render, and a finished request's bytes return to the budget."""
    import ctypes as C
    from yune_gb300 import _native as N
    from yune_gb300.core import cfg_struct
    s = scenes.c1(8, 8, level=3)
    with Renderer(0) as r:
        sid = r.upload(s)
        L = r.L
        bc = N.BatchCfg(2048, 2, 2, 1, 64, r.scene_depth(sid) + 2, 0, 1, 0)
        sc = N.ServeCfg(24 * 20 * 16 + 64, -1, 1, bc)
        h = C.c_void_p()
        N.check(L.yc_serve_create(r.h, C.byref(sc), C.byref(h)), "create")
        seeds = scenes.pass_seeds(9, 3)
        d = N.RequestDesc()
        C.memmove(C.byref(d.cam), s.cam.ctypes.data, C.sizeof(N.Cam))
        d.cfg = cfg_struct(s.cfg)
        d.scene_id, d.width, d.height, d.n_pass, d.seeds_host = sid, 24, 20, 3, seeds.ctypes.data
        ids = []
        for _ in range(2):
            rid, st = C.c_int64(), C.c_int32()
            N.check(L.yc_serve_submit(h, C.byref(d), C.byref(rid), C.byref(st)), "submit")
            ids.append((rid.value, st.value))
        assert [st for _, st in ids] == [N.REQ_RUNNING, N.REQ_WAITING]   # one fits the budget at a time
        run, wait = C.c_int32(), C.c_int32()
        info = N.RequestInfo()
        for _ in range(10000):
            N.check(L.yc_serve_step(h, 1, C.byref(run), C.byref(wait)), "step")
            N.check(L.yc_serve_info(h, ids[0][0], C.byref(info)), "info")
            if info.state == N.REQ_DONE:
                break
        assert info.state == N.REQ_DONE and info.pixels_done == info.pixels_total == 24 * 20
        assert 0 <= info.submit_s <= info.admit_s <= info.finish_s
        out = np.zeros((20, 24, 4), np.float32)
        N.check(L.yc_serve_read(h, ids[0][0], out.ctypes.data), "read")
        N.check(L.yc_serve_step(h, 0, C.byref(run), C.byref(wait)), "step")
        N.check(L.yc_serve_info(h, ids[1][0], C.byref(info)), "info")
        assert info.state == N.REQ_WAITING            # the first still holds its bytes (kept result)
        N.check(L.yc_serve_release(h, ids[0][0]), "release")
        N.check(L.yc_serve_step(h, 0, C.byref(run), C.byref(wait)), "step")
        N.check(L.yc_serve_info(h, ids[1][0], C.byref(info)), "info")
        assert info.state == N.REQ_RUNNING and wait.value == 0
        N.check(L.yc_serve_destroy(h), "destroy")
        r.set_camera(s.cam)
        aid = r.alloc_accum(24, 20)
        r.render_passes(sid, aid, seeds, reset_first=1, cfg=s.cfg)
        assert np.array_equal(out.view(np.int32), r.read_accum(aid).view(np.int32))


@pytest.mark.parametrize("tree", [0, 1, 2])
def test_layout_bytes_are_the_upload_bytes_in_every_tree_mode(tree):
    """The admission estimate (yc_scene_layout on the host) is what the upload holds on the
    device (yc_scene_bytes), in each layout a renderer can be set to."""
    s = scenes.c1(8, 8, level=4)
    with Renderer(0) as r:
        r.set_tree_mode(tree)
        sid = r.upload(s)
        assert r.scene_bytes(sid) == scenes.device_bytes(s, tree_mode=tree)
