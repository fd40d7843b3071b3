"""The server's host logic without a GPU: admission by HBM budget, rejection of requests
larger than the budget or beyond the waiting-queue limit, cancellation of waiting and
of admitted requests (the engine is a fake that completes a fixed number of pixels per
launch and records cancellations)."""
import itertools

import pytest

from yune_gb300 import scenes, serve


class FakeBatch:
    def __init__(self, renderer, **kw):
        self.jobs = []          # [done, total, cancelled]
        self.cancelled = []
        self.per_launch = 64

    def add_job(self, sid, accum, cam, seeds, cfg):
        w, h = self.r_sizes[accum]
        self.jobs.append([0, w * h, False])
        return len(self.jobs) - 1

    def run(self, max_launches=0):
        for j in self.jobs:
            if j[0] < j[1]:
                j[0] = j[1] if j[2] else min(j[1], j[0] + self.per_launch)

    def progress(self, job):
        return self.jobs[job][0], self.jobs[job][1]

    def cancel(self, job):
        self.jobs[job][2] = True
        self.cancelled.append(job)

    def close(self):
        pass


class FakeRenderer:
    def __init__(self):
        self.sizes = {}
        self.ids = itertools.count()
        self.freed = []

    def upload(self, s):
        return next(self.ids)

    def scene_depth(self, sid):
        return 8

    def alloc_accum(self, w, h):
        a = next(self.ids)
        self.sizes[a] = (w, h)
        return a

    def free_accum(self, a):
        self.freed.append(a)

    def read_accum(self, a):
        return None


class Clock:
    """Each call advances time by dt: the server loop sees time pass per launch."""
    def __init__(self, dt=0.01):
        self.t, self.dt = 0.0, dt

    def __call__(self):
        self.t += self.dt
        return self.t


@pytest.fixture
def server(monkeypatch):
    def make(budget, max_queue=None):
        r = FakeRenderer()

        def fake_batch(renderer, **kw):
            b = FakeBatch(renderer, **kw)
            b.r_sizes = r.sizes
            return b
        monkeypatch.setattr(serve, "Batch", fake_batch)
        resident = [scenes.SceneData(None, None, None, None, 8, None, 8, 8, 1, {}, "fake")]
        return serve.Server(r, resident, hbm_budget=budget, max_queue=max_queue), r
    return make


def _req(t, w, h, spp=2, cancel=None):
    return serve.Request(t, 0, w, h, spp, cancel_after=cancel)


def test_admission_by_budget_and_rejections(server):
    srv, r = server(budget=2 * (16 * 16 * 16 + 8), max_queue=1)
    reqs = [_req(0.0, 16, 16), _req(0.0, 16, 16), _req(0.0, 16, 16), _req(0.0, 16, 16), _req(0.0, 64, 64)]
    done = srv.run(reqs, clock=Clock())
    st = [q.status for q in done]
    # two fit the budget, one waits, the fourth finds the queue full; 64x64 exceeds the budget
    assert st.count("done") == 3
    assert st.count("rejected: queue full") == 1
    assert st.count("rejected: larger than the whole HBM budget") == 1
    assert srv.max_in_use <= srv.budget and srv.max_in_flight == 2
    assert srv.in_use == 0 and len(r.freed) == 3


def test_cancel_waiting_and_admitted(server):
    srv, r = server(budget=16 * 16 * 16 + 8)   # one request at a time
    a = _req(0.0, 16, 16, cancel=0.03)   # admitted, cancelled while it runs
    b = _req(0.0, 16, 16, cancel=0.02)   # waits behind a, cancelled before admission
    c = _req(0.0, 16, 16)
    done = srv.run([a, b, c], clock=Clock())
    assert [q.status for q in done] == ["cancelled", "cancelled", "done"]
    assert srv.batch.cancelled == [a.job]     # only the admitted one reached the engine
    assert b.job == -1 and b.accum == -1
    assert a.accum in r.freed and c.accum in r.freed and srv.in_use == 0
    assert a.done < c.done


def test_resident_scenes_checked_against_a_scene_budget(monkeypatch):
    """The resident scenes' device bytes (yc_scene_layout, computed on the host) are
    checked before any upload; over budget, the server refuses to start."""
    monkeypatch.setattr(serve, "Batch", lambda renderer, **kw: FakeBatch(renderer, **kw))
    resident = [scenes.c0(16, 16), scenes.c1(16, 16, level=3)]
    need = sum(scenes.device_bytes(s) for s in resident)
    assert need > 0
    r = FakeRenderer()
    with pytest.raises(ValueError, match="scene budget"):
        serve.Server(r, resident, hbm_budget=1 << 20, scene_budget=need - 1)
    assert next(r.ids) == 0                               # nothing was uploaded
    srv = serve.Server(FakeRenderer(), resident, hbm_budget=1 << 20, scene_budget=need)
    assert srv.scene_bytes == need
