"""Reference node arrays with chosen leaf boxes, for the repack tests.

A complete binary tree in breadth-first (heap) order: node i has its children at 2i + 1
and 2i + 2, the n leaves are the last n nodes, each holding one triangle. The repack keeps
only the leaves (their boxes, triangles and tie-break ranks) and builds its own SAH
hierarchy above them, so the leaf boxes choose which of its paths run:

- "coincident": every leaf box equal (every split falls back to halving the list);
- "grid": boxes on a small integer grid, zeros of either sign (equal split costs, -0 and
  +0 in one min / max);
- "random": uniform boxes.
"""
from types import SimpleNamespace

import numpy as np

from yune_gb300 import scenes
from yune_gb300.layouts import BVH_NODE, TRIANGLE


def leaf_boxes(n, kind, seed=0):
    rng = np.random.default_rng(seed)
    if kind == "coincident":
        lo = np.tile(np.float32([0.25, -0.5, 1.0]), (n, 1))
        hi = lo + np.float32(0.125)
    elif kind == "grid":
        lo = rng.integers(-4, 5, (n, 3)).astype(np.float32)
        hi = lo + rng.integers(0, 3, (n, 3)).astype(np.float32)
        neg = rng.random((n, 3)) < 0.5
        lo[(lo == 0) & neg] = np.float32(-0.0)
        hi[(hi == 0) & ~neg] = np.float32(-0.0)
    elif kind == "random":
        lo = rng.random((n, 3), np.float32) * np.float32(8.0) - np.float32(4.0)
        hi = lo + rng.random((n, 3), np.float32) * np.float32(0.5)
    else:
        raise ValueError(kind)
    return lo.astype(np.float32), hi.astype(np.float32)


def leaf_scene(n, kind, seed=0):
    """A scene (tris, mats, lights, nodes) of n one-triangle leaves with kind's boxes;
    the materials, lights and camera are the Cornell box's."""
    lo, hi = leaf_boxes(n, kind, seed)
    tris = np.zeros(n, TRIANGLE)
    tris["v1"][:, :3] = lo
    tris["v2"][:, :3] = hi
    tris["v3"][:, :3] = np.stack([lo[:, 0], hi[:, 1], lo[:, 2]], 1)
    for k in ("vn1", "vn2", "vn3"):
        tris[k][:, 2] = 1.0
    nodes = np.zeros(2 * n - 1, BVH_NODE)
    first_leaf = n - 1
    nodes["child_idx"][:first_leaf] = 2 * np.arange(first_leaf) + 1
    nodes["vert_len"][:first_leaf] = -1
    nodes["child_idx"][first_leaf:] = -1
    nodes["vert_len"][first_leaf:] = 1
    nodes["vert_list"][first_leaf:, 0] = np.arange(n)
    nodes["p_min"][first_leaf:, :3] = lo
    nodes["p_max"][first_leaf:, :3] = hi
    b = first_leaf   # interior boxes: unions, bottom up, nodes [a, b) at once (their children lie at b or above)
    while b > 0:
        a = b // 2
        i = np.arange(a, b)
        nodes["p_min"][a:b] = np.minimum(nodes["p_min"][2 * i + 1], nodes["p_min"][2 * i + 2])
        nodes["p_max"][a:b] = np.maximum(nodes["p_max"][2 * i + 1], nodes["p_max"][2 * i + 2])
        b = a
    base = scenes.c0(16, 16)
    return SimpleNamespace(tris=tris, mats=base.mats, lights=base.lights, nodes=nodes, cam=base.cam)
