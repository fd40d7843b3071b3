"""The batch autotuner's search on the CPU, with a fake calibration clock."""
from yune_gb300 import autotune


class _FakeRenderer:
    def __init__(self):
        self.live = 0

    def alloc_accum(self, w, h):
        self.live += 1
        return self.live

    def free_accum(self, a):
        self.live -= 1


def test_coordinate_search_finds_the_separable_optimum(monkeypatch):
    seen = []

    def clock(renderer, jobs, shape, cap, accs, passes=1):
        seen.append(shape.kwargs())
        return (abs(shape.pool_paths - (1 << 20)) / 1e5 + abs(shape.rounds_per_launch - 16)
                + abs(shape.logic_blocks_per_sm - 2))

    monkeypatch.setattr(autotune, "_calibrate", clock)
    r = _FakeRenderer()
    best, trials = autotune.tune(r, [(0, None, [1], None)] * 3, [(1920, 1080)] * 3)
    assert best == autotune.BatchShape(1 << 20, 16, 2, 1 << 16, 2)
    assert len(trials) == len(seen) and r.live == 0   # scratch accumulators released


def test_pool_never_exceeds_the_pixels_in_the_mix(monkeypatch):
    monkeypatch.setattr(autotune, "_calibrate", lambda r, j, shape, c, a, passes=1: 1.0 / shape.pool_paths)
    best, trials = autotune.tune(_FakeRenderer(), [(0, None, [1], None)], [(256, 256)])
    assert best.pool_paths == 1 << 16
    assert all(t.pool_paths <= 1 << 16 for t, _ in trials)


def test_small_mixes_calibrate_over_several_passes():
    """A frame smaller than the largest pool is calibrated over enough passes to fill that
    pool four times (at most 16); a large mix needs one pass."""
    assert autotune.calibration_passes(1024 * 1024) == 16
    assert autotune.calibration_passes(8 << 20) == 2
    assert autotune.calibration_passes(60_000_000) == 1
