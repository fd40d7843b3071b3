"""The host replay of the traversal (yc_walk_counts), which counts the algorithmic work
of the traversal roofline: one ray at a time in the device walk's order, without a warp's
speculation. Its results must be the reference's (closest triangle and t bit for bit, the
any-hit verdict), in every tree mode; and the oracle's record of the rays a pass
walks must hold the rays the core walks (camera rays: one per pixel)."""
import numpy as np
import pytest

from oracle import oracle_py as O
from yune_gb300 import _native as N
from yune_gb300 import scenes, workloads


@pytest.mark.parametrize("tree", [0, 1, 2])
@pytest.mark.parametrize("name", ["c0", "c1"])
def test_replay_hits_equal_the_reference(name, tree):
    s = scenes.c0(32, 32) if name == "c0" else scenes.c1(32, 32, level=4)
    rays = O.seeded_rays(s, 20000, seed=5)
    boxes, tris, tri, t = scenes.walk_counts(s, rays, any_hit=False, tree_mode=tree)
    ot, ol, ott, ov = O.trace(s, rays)
    assert ov.sum() == 0
    walked = ol < 0   # (a light in front settles the ray before any walk)
    assert np.array_equal(tri[walked], ot[walked])
    assert np.array_equal(t[walked].view(np.int32), ott[walked].view(np.int32))
    assert boxes > 0 and tris > 0
    seg = rays.copy()
    seg[:, 8] = np.where(np.isfinite(ott), ott * np.float32(1.001), np.float32(0.6))
    _, _, atri, _ = scenes.walk_counts(s, seg, any_hit=True, tree_mode=tree)
    assert np.array_equal(atri >= 0, O.trace(s, seg, any_hit=True)[0] >= 0)


def test_reference_tree_needs_more_boxes_than_the_sah_tree():
    s = scenes.c1(32, 32, level=5)
    rays = O.seeded_rays(s, 5000, seed=2)
    b0, _, _, _ = scenes.walk_counts(s, rays, tree_mode=0)
    b1, _, _, _ = scenes.walk_counts(s, rays, tree_mode=1)
    assert b1 < b0


def test_recorded_rays_of_a_pass():
    s = workloads.mixed_scene(20000, 3, 64, 48, 1, scenes.default_cfg(max_depth=16, mis_lobe_fix=0))
    rec = O.record_rays(s, 777, s.cfg, (10, 14))
    kinds = np.bincount(rec[:, 7].astype(int), minlength=4)
    assert kinds[0] == 4 * 64                         # one camera ray per pixel of the rows
    assert kinds[1] > 0 and kinds[2] > 0
    assert np.all(np.isfinite(rec[:, :6])) and np.all(rec[:, 6] > 0)
    # the closest-hit replay of the recorded camera rays finds their triangles
    cam = O.rays9_of(rec[rec[:, 7] == 0])
    _, _, tri, _ = scenes.walk_counts(s, cam)
    assert (tri >= 0).mean() > 0.5


def test_replay_refuses_an_unknown_tree_mode():
    s = scenes.c0(8, 8)
    with pytest.raises(N.YuneError):
        scenes.walk_counts(s, O.seeded_rays(s, 10), tree_mode=7)
