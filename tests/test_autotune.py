"""The batch tuner's search on the CPU (yc_tune_search, the search of yc_batch_tune with a
clock supplied by the caller): one parameter at a time, each keeping its best value, a
second sweep when the first moved, the pool bounded by the mix's pixels."""
from yune_gb300 import autotune

START = autotune.BatchShape()


def test_coordinate_search_finds_the_separable_optimum():
    seen = []

    def clock(shape):
        seen.append(shape.kwargs())
        return (abs(shape.pool_paths - (1 << 20)) / 1e5 + abs(shape.rounds_per_launch - 16)
                + abs(shape.logic_blocks_per_sm - 2) + abs(shape.trace_block - 256) / 64.0)

    best, trials = autotune.search(START, 3 * 1920 * 1080, clock)
    assert best == autotune.BatchShape(1 << 20, 16, 2, 1 << 16, 2, 0, 256)
    assert len(trials) == len(seen)
    assert len({tuple(sorted(k.items())) for k in seen}) == len(seen)   # no shape timed twice


def test_pool_never_exceeds_the_pixels_in_the_mix():
    best, trials = autotune.search(START, 256 * 256, lambda shape: 1.0 / shape.pool_paths)
    assert best.pool_paths == 1 << 16
    assert all(t.pool_paths <= 1 << 16 for t, _ in trials)


def test_trace_block_is_searched_and_a_second_sweep_follows_a_move():
    def clock(shape):   # rewards 64-thread trace blocks, then 4 groups once blocks are 64 wide
        return (shape.trace_block != 64) * 10 + (shape.trace_block == 64 and shape.groups != 4) * 5

    best, trials = autotune.search(START, 8 << 20, clock)
    assert best.trace_block == 64 and best.groups == 4
    assert {t.trace_block for t, _ in trials} >= {64, 128, 256}


def test_stack_split_is_searched():
    """stack_smem (walk-stack entries kept in shared memory) is a search dimension: 8, 12,
    16 or the whole stack (64)."""
    best, trials = autotune.search(START, 8 << 20, lambda shape: abs(shape.stack_smem - 8))
    assert best.stack_smem == 8
    assert {t.stack_smem for t, _ in trials} >= {8, 12, 16, 64}


def test_small_mixes_calibrate_over_several_passes():
    """A frame smaller than the largest pool is calibrated over enough passes to fill that
    pool four times (at most 16); a large mix needs one pass."""
    assert autotune.calibration_passes(1024 * 1024) == 16
    assert autotune.calibration_passes(8 << 20) == 2
    assert autotune.calibration_passes(60_000_000) == 1


def test_groups_and_trace_share_are_searched_together():
    """More slot groups pay only when each group's traversal leaves room on the SMs for
    the others (trace_share below 100): the two are one search dimension, so an optimum
    that neither reaches alone (4 groups at 50%, where 4 groups at 100% and 2 groups at
    50% are both worse than the start) is found."""
    def clock(shape):
        if shape.groups == 4 and shape.trace_share == 50:
            return 1.0
        return 2.0 + (shape.groups != 2) + (shape.trace_share != 100)

    best, trials = autotune.search(START, 8 << 20, clock)
    assert (best.groups, best.trace_share) == (4, 50)
    assert {(t.groups, t.trace_share) for t, _ in trials} >= {(1, 100), (2, 100), (4, 100), (2, 50), (4, 50),
                                                                 (8, 50), (4, 25), (8, 25)}
