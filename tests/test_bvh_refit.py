"""yh_bvh_refit: the bottom-up box pass of BVH::createBVH (BVH::resizeBvh,
src/BVH.cpp:218-247) run on moved triangles. On unmoved triangles it leaves the node
array unchanged bit for bit; on moved ones every box is the union the reference pass
gives and traversal through the refitted tree finds the same closest hits as testing
every triangle (the oracle's brute force, udpt.cl:240-286 with bvh_size 0). CPU only."""
import dataclasses

import numpy as np
import pytest

from oracle import oracle_py as O
from yune_gb300 import _native as N
from yune_gb300 import scenes


def _moved(s, seed=4):
    """s with every vertex displaced by a smooth field of the vertex position (shared
    vertices move together, so the mesh stays closed), normals kept."""
    t = s.tris.copy()
    rng = np.random.default_rng(seed)
    k = rng.uniform(3.0, 9.0, size=3)
    ph = rng.uniform(0.0, 6.3, size=3)
    for f in ("v1", "v2", "v3"):
        p = t[f][:, :3].astype(np.float64)
        d = 0.04 * np.sin(k * p[:, [1, 2, 0]] + ph) + np.array([0.03, -0.02, 0.05])
        t[f][:, :3] = (p + d).astype(np.float32)
    return dataclasses.replace(s, tris=t)


def _padded_boxes(t):
    v = np.stack([t["v1"][:, :3], t["v2"][:, :3], t["v3"][:, :3]])
    lo = np.minimum(v[0], np.minimum(v[1], v[2]))
    hi = np.maximum(v[0], np.maximum(v[1], v[2]))
    hi = np.where(hi - lo == np.float32(0), hi + np.float32(0.2), hi)   # TriangleCPU.cpp:63-67
    return lo, hi


@pytest.mark.parametrize("make", [lambda: scenes.c0(16, 16), lambda: scenes.c1(16, 16, level=4),
                                  lambda: scenes.c1(16, 16, level=7)], ids=["c0", "c1_l4", "c1_l7"])
def test_refit_of_unmoved_scene_is_the_build(make):
    s = make()
    out = scenes.refit_bvh(s.tris, s.nodes)
    assert out.tobytes() == s.nodes.tobytes()


def test_refit_boxes_are_the_reference_pass():
    s = scenes.c1(16, 16, level=4)
    m = _moved(s)
    nodes = scenes.refit_bvh(m.tris, s.nodes)
    lo, hi = _padded_boxes(m.tris)
    leaf = nodes["vert_len"] > 0
    for j in np.nonzero(leaf)[0]:
        ids = nodes["vert_list"][j, :nodes["vert_len"][j]]
        assert np.array_equal(nodes["p_min"][j, :3], lo[ids].min(axis=0))
        assert np.array_equal(nodes["p_max"][j, :3], hi[ids].max(axis=0))
        assert nodes["p_min"][j, 3] == 1.0 and nodes["p_max"][j, 3] == 1.0
    inner = ~leaf & (nodes["child_idx"] > 0)
    for j in np.nonzero(inner)[0]:
        c = nodes["child_idx"][j]
        assert np.array_equal(nodes["p_min"][j, :3], np.minimum(nodes["p_min"][c, :3], nodes["p_min"][c + 1, :3]))
        assert np.array_equal(nodes["p_max"][j, :3], np.maximum(nodes["p_max"][c, :3], nodes["p_max"][c + 1, :3]))
    empty = ~leaf & ~inner
    assert np.array_equal(nodes[empty].tobytes(), s.nodes[empty].tobytes())
    # only boxes change
    for f in ("child_idx", "vert_len", "vert_list"):
        assert np.array_equal(nodes[f], s.nodes[f])


def test_refitted_tree_finds_the_brute_force_hits():
    s = scenes.c1(16, 16, level=4)
    m = _moved(s)
    refit = dataclasses.replace(m, nodes=scenes.refit_bvh(m.tris, s.nodes))
    brute = dataclasses.replace(m, nodes=s.nodes[:0])
    rays = O.seeded_rays(m, 20000, seed=8)
    tri_a, light_a, t_a, ov = O.trace(refit, rays)
    tri_b, light_b, t_b, _ = O.trace(brute, rays)
    assert ov.sum() == 0
    assert np.array_equal(light_a, light_b)
    assert np.array_equal(t_a.view(np.int32), t_b.view(np.int32))
    # the same triangle unless two triangles are hit at exactly the same distance (a
    # shared edge), where the visiting order decides (none among these rays)
    diff = np.nonzero(tri_a != tri_b)[0]
    assert len(diff) <= 2, diff
    # the stale build would miss moved geometry: the refit is what makes the hits right
    stale = dataclasses.replace(m, nodes=s.nodes)
    _, _, t_s, _ = O.trace(stale, rays)
    assert not np.array_equal(t_s.view(np.int32), t_b.view(np.int32))


def test_refit_rejects_malformed_arrays():
    s = scenes.c1(16, 16, level=3)
    L = N.lib()
    bad = s.nodes.copy()
    j = int(np.nonzero(bad["vert_len"] > 0)[0][0])
    bad["vert_list"][j, 0] = len(s.tris)   # a triangle that does not exist
    with pytest.raises(N.YuneError) as e:
        scenes.refit_bvh(s.tris, bad)
    assert e.value.code == N.YH_E_RANGE
    bad = s.nodes.copy()
    k = int(np.nonzero((bad["vert_len"] <= 0) & (bad["child_idx"] > 0))[0][-1])
    bad["child_idx"][k] = k   # a child that does not come after its parent
    with pytest.raises(N.YuneError) as e:
        scenes.refit_bvh(s.tris, bad)
    assert e.value.code == N.YH_E_RANGE
    bad = s.nodes.copy()
    bad["vert_len"][j] = 11
    with pytest.raises(N.YuneError) as e:
        scenes.refit_bvh(s.tris, bad)
    assert e.value.code == N.YH_E_RANGE
    assert L.yh_bvh_refit(None, 3, None, 0) == N.YH_E_INVALID
    assert L.yh_bvh_refit(None, 0, None, 0) == 0   # nothing to do
