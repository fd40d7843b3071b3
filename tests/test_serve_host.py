"""The server's admission rules without a GPU (yc_admission_*, the host-only object the
request server of the C-ABI admits with): admission by HBM budget in arrival order,
rejection of requests larger than the budget or beyond the waiting-queue limit,
cancellation of waiting and of admitted requests, and the resident-scene budget checked
before anything is uploaded."""
import pytest

from yune_gb300 import _native as N
from yune_gb300 import scenes, serve

REQ = 16 * 16 * 16 + 8   # a 16 x 16 request of two passes


def test_admission_by_budget_and_rejections():
    a = serve.Admission(2 * REQ, max_queue=1)
    got = [a.submit(REQ) for _ in range(4)] + [a.submit(64 * 64 * 16 + 8)]
    # two fit the budget, one waits, the fourth finds the queue full; 64x64 exceeds the budget
    assert [s for _, s in got] == [N.REQ_RUNNING, N.REQ_RUNNING, N.REQ_WAITING, N.REQ_REJECTED_QUEUE,
                                   N.REQ_REJECTED_BUDGET]
    assert a.usage() == (2 * REQ, 1, 2)
    assert a.next() == -1                      # nothing fits until a running request finishes
    assert a.finish(got[0][0]) == N.REQ_DONE
    assert a.next() == got[2][0] and a.state(got[2][0]) == N.REQ_RUNNING
    assert a.usage() == (2 * REQ, 0, 2)
    for t in (got[1][0], got[2][0]):
        a.finish(t)
    assert a.usage() == (0, 0, 0)
    with pytest.raises(N.YuneError):
        a.finish(got[3][0])                     # a rejected request holds nothing


def test_cancel_waiting_and_admitted():
    a = serve.Admission(REQ)                    # one request at a time
    ra, _ = a.submit(REQ)
    rb, sb = a.submit(REQ)
    rc, _ = a.submit(REQ)
    assert sb == N.REQ_WAITING
    assert a.cancel(rb) == N.REQ_CANCELLED      # dropped while it waits
    assert a.cancel(ra) == N.REQ_CANCELLING     # stops in the engine, still holds its bytes
    assert a.usage() == (REQ, 1, 1) and a.next() == -1
    assert a.finish(ra) == N.REQ_CANCELLED      # its work drained: bytes released
    assert a.next() == rc and a.state(rb) == N.REQ_CANCELLED
    assert a.cancel(rb) == N.REQ_CANCELLED      # cancelling twice changes nothing


def test_oldest_waiting_request_is_never_overtaken():
    a = serve.Admission(4 * REQ)
    r0, _ = a.submit(3 * REQ)
    big, s = a.submit(2 * REQ)                  # waits: 3 + 2 > 4
    small, s2 = a.submit(REQ)                   # would fit, but queues behind `big`
    assert (s, s2) == (N.REQ_WAITING, N.REQ_WAITING)
    assert a.next() == -1
    a.finish(r0)
    assert a.next() == big and a.next() == small and a.usage() == (3 * REQ, 0, 2)


def test_unbounded_queue_and_budget_edges():
    a = serve.Admission(REQ)
    states = [a.submit(REQ)[1] for _ in range(50)]
    assert states[0] == N.REQ_RUNNING and set(states[1:]) == {N.REQ_WAITING}
    assert a.submit(REQ + 1)[1] == N.REQ_REJECTED_BUDGET
    assert a.submit(0)[1] == N.REQ_WAITING      # behind the others, though it needs nothing


def test_resident_scenes_checked_against_a_scene_budget():
    """The resident scenes' device bytes (yc_scene_layout, computed on the host) are
    checked before any upload; over budget, the server refuses to start."""
    class NoUploads:
        tree_mode = 1

        def upload(self, s):
            raise AssertionError("nothing may be uploaded")

    resident = [scenes.c0(16, 16), scenes.c1(16, 16, level=3)]
    need = sum(scenes.device_bytes(s) for s in resident)
    assert need > 0
    with pytest.raises(ValueError, match="scene budget"):
        serve.Server(NoUploads(), resident, hbm_budget=1 << 20, scene_budget=need - 1)
    r = NoUploads()
    r.tree_mode = 2                              # four-child nodes take other bytes
    need4 = sum(scenes.device_bytes(s, tree_mode=2) for s in resident)
    with pytest.raises(ValueError, match="scene budget"):
        serve.Server(r, resident, hbm_budget=1 << 20, scene_budget=need4 - 1)
