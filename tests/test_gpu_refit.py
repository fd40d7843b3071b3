"""Refit of an uploaded scene on the device (yc_refit_scene) for moving geometry: after the
triangles move, a render equals the oracle's on the moved triangles with the reference's
node array refitted by BVH::resizeBvh (yh_bvh_refit), in every tree mode; unmoved
triangles leave the render unchanged."""
import dataclasses

import numpy as np
import pytest

from oracle import oracle_py as O
from yune_gb300 import scenes
from yune_gb300.core import Renderer

pytestmark = pytest.mark.gpu


def _moved(tris):
    """Every vertex moved by a smooth function of its position (shared vertices stay shared)."""
    out = tris.copy()
    for v in ("v1", "v2", "v3"):
        p = out[v][:, :3].astype(np.float64)
        d = np.stack([0.02 * np.sin(9.0 * p[:, 1]), 0.03 * np.sin(7.0 * p[:, 0] + 1.0), 0.015 * np.cos(5.0 * p[:, 2])],
                     axis=1)
        moving = np.abs(p).max(axis=1) < 0.45          # the walls stay put
        out[v][:, :3] = np.where(moving[:, None], p + d, p).astype(np.float32)
    return out


def _render(r, s, sid, seeds):
    r.set_camera(s.cam)
    aid = r.alloc_accum(s.width, s.height)
    r.reset_stats()
    r.render_passes(sid, aid, seeds, reset_first=1, cfg=s.cfg)
    img, st = r.read_accum(aid), r.stats()
    r.free_accum(aid)
    return img, st


def _oracle(s, seeds):
    ref = np.zeros((s.height, s.width, 4), np.float32)
    rays = 0
    for k, sd in enumerate(seeds):
        rays += O.render(s, ref, sd, 1 if k == 0 else 0, s.cfg)["rays"]
    return ref, rays


@pytest.mark.parametrize("tree", [0, 1, 2])
def test_refit_render_equals_the_refitted_reference(tree):
    s = scenes.c1(40, 32, level=4)
    seeds = scenes.pass_seeds(51, 2)
    moved = _moved(s.tris)
    assert not np.array_equal(moved, s.tris)
    with Renderer(0) as r:
        r.set_tree_mode(tree)
        sid = r.upload(s)
        r.set_tree_mode(1)
        r.refit(sid, moved)
        img, st = _render(r, s, sid, seeds)
        assert st["stack_overflow"] == 0
        r.refit(sid, s.tris)                       # and back: the original render
        back, _ = _render(r, s, sid, seeds)
        fresh_sid = r.upload(s)
        fresh, _ = _render(r, s, fresh_sid, seeds)
    sm = dataclasses.replace(s, tris=moved, nodes=scenes.refit_bvh(moved, s.nodes))
    ref, rays = _oracle(sm, seeds)
    assert np.array_equal(img.view(np.int32), ref.view(np.int32))
    assert st["rays"] == rays
    assert np.array_equal(back.view(np.int32), fresh.view(np.int32))


def test_refit_without_a_bvh_and_argument_checks():
    s = scenes.c0(24, 20)
    s.nodes = s.nodes[:0]                          # brute force over every triangle
    seeds = scenes.pass_seeds(52, 2)
    moved = _moved(s.tris)
    from yune_gb300 import _native as N
    with Renderer(0) as r:
        sid = r.upload(s)
        r.refit(sid, moved)
        img, _ = _render(r, s, sid, seeds)
        with pytest.raises(N.YuneError):
            r.refit(sid, moved[:-1])               # another triangle count
        bad = moved.copy()
        bad["matID"][0] = 99
        with pytest.raises(N.YuneError):
            r.refit(sid, bad)
    ref, _ = _oracle(dataclasses.replace(s, tris=moved), seeds)
    assert np.array_equal(img.view(np.int32), ref.view(np.int32))
