"""The upload's repack on the device (YC_OPT_REPACK 1, the default for tree mode 1) writes
the bytes of the host repack: the digest of the uploaded arrays (yc_scene_digest) equals
yc_scene_layout's for the same inputs, with the same depth and device bytes, on the
procedural scenes and on node arrays whose leaf boxes steer the SAH split into its corner
cases (coincident centroids, equal costs, zeros of both signs), at sizes that take the
shared-memory subtree builds alone and the level-by-level splits above them."""
import numpy as np
import pytest

import leafgen
from oracle import oracle_py as O
from yune_gb300 import scenes
from yune_gb300.core import Renderer

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def r():
    with Renderer(0) as rr:
        yield rr


def _no_bvh():
    s = scenes.c0(16, 16)
    s.nodes = s.nodes[:0]
    return s


def _no_triangles():
    s = scenes.c0(16, 16)
    s.tris, s.nodes = s.tris[:0], s.nodes[:0]
    return s


def _one_reachable_leaf():
    # an interior root whose second child the reference never queues (vert_len 0, no children)
    s = leafgen.leaf_scene(2, "random", 8)
    s.nodes["vert_len"][2] = 0
    s.nodes["child_idx"][2] = -2
    return s


CASES = {
    # scenes the upload repacks on the host whatever the option (no BVH, no triangles, a
    # leaf at the root, fewer than two reachable leaves)
    "no_bvh": _no_bvh,
    "no_triangles": _no_triangles,
    "root_leaf": lambda: leafgen.leaf_scene(1, "random", 9),
    "one_reachable_leaf": _one_reachable_leaf,
    "c0": lambda: scenes.c0(16, 16),
    "c1_l5": lambda: scenes.c1(16, 16, level=5),
    "c1_l7": lambda: scenes.c1(16, 16, level=7),
    "two_leaves": lambda: leafgen.leaf_scene(2, "random", 1),
    "three_leaves": lambda: leafgen.leaf_scene(3, "grid", 2),
    "small_max": lambda: leafgen.leaf_scene(512, "random", 3),
    "small_max_plus_1": lambda: leafgen.leaf_scene(513, "grid", 4),
    "coincident": lambda: leafgen.leaf_scene(3000, "coincident", 5),
    "grid": lambda: leafgen.leaf_scene(140000, "grid", 6),
    "random": lambda: leafgen.leaf_scene(140000, "random", 7),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_device_repack_equals_host_repack(r, case):
    s = CASES[case]()
    lay = scenes.layout(s, 1)
    r.set_tree_mode(1)
    got = {}
    for mode in (1, 0):
        r.set_repack(mode)
        sid = r.upload(s)
        got[mode] = (r.scene_digest(sid), r.scene_depth(sid), r.scene_bytes(sid))
        r.release(sid)
    r.set_repack(1)
    assert got[1] == got[0]
    assert got[1] == (lay["digest"], lay["depth"], lay["device_bytes"])


def test_render_after_device_repack_equals_oracle(r):
    """A pass over the device-repacked glass sphere gives the oracle's bits, as over the
    host-repacked one."""
    s = scenes.c1(40, 32, level=5)
    seeds = scenes.pass_seeds(53, 2)
    r.set_tree_mode(1)
    r.set_camera(s.cam)
    out = []
    for mode in (1, 0):
        r.set_repack(mode)
        sid = r.upload(s)
        aid = r.alloc_accum(40, 32)
        r.render_passes(sid, aid, seeds, reset_first=1, cfg=s.cfg)
        out.append(r.read_accum(aid))
        r.free_accum(aid)
        r.release(sid)
    r.set_repack(1)
    ref = np.zeros((32, 40, 4), np.float32)
    for k, sd in enumerate(seeds):
        O.render(s, ref, sd, 1 if k == 0 else 0, s.cfg)
    for img in out:
        assert np.array_equal(img.view(np.int32), ref.view(np.int32))


def test_repack_option_checked(r):
    from yune_gb300 import _native as N
    assert r.L.yc_set_option(r.h, 10, 2) == N.YC_E_INVALID
    assert r.L.yc_set_option(r.h, 10, -1) == N.YC_E_INVALID
