"""yc_scene_layout: the device layout yc_upload_scene builds (the repack of the
reference node array into two- or four-child nodes, the 48-byte triangle stream and
the shading records), computed on the host without a device. Its digest must not depend
on the number of host threads the repack runs on, and malformed inputs are refused as
the upload refuses them. CPU only."""
import ctypes as C

import numpy as np
import pytest

import leafgen
from yune_gb300 import _native as N
from yune_gb300 import scenes
from yune_gb300.layouts import MATERIAL, QUAD_LIGHT, ptr


def layout(tris, n_mat, nodes, tree=1):
    out = N.SceneLayout()
    N.check(N.lib().yc_scene_layout(ptr(tris), len(tris), n_mat, ptr(nodes), len(nodes), tree, C.byref(out)),
            "yc_scene_layout")
    return out


@pytest.fixture(scope="module")
def big():
    # 327,714 triangles, leaves of up to 4: about 82K leaves, so the repack's SAH build
    # over the leaves splits subtrees onto threads
    s = scenes.c1(16, 16, level=7)
    nodes, _ = scenes.build_bvh(s.tris, 20, 4)
    return s, nodes


@pytest.mark.parametrize("tree", [0, 1, 2])
def test_layout_digest_independent_of_host_threads(big, tree):
    s, nodes = big
    L = N.lib()
    got = {}
    try:
        for th in (1, 2, 5, 0):
            assert L.yh_set_host_threads(th) == 0
            lay = layout(s.tris, len(s.mats), nodes, tree)
            got[th] = (lay.digest, lay.device_bytes, lay.depth, lay.wide)
    finally:
        L.yh_set_host_threads(0)
    assert len(set(got.values())) == 1, got
    assert got[0][3] == (1 if tree == 2 else 0)


def test_layout_sizes(big):
    s, nodes = big
    lay = layout(s.tris, len(s.mats), nodes, 1)
    # 48-byte stream record per triangle, 64-byte shading record per triangle, 64-byte
    # two-child nodes; materials as uploaded with their 8-byte Oren-Nayar constants, and
    # the 16-light table
    assert lay.stream_bytes == 48 * s.n_tri
    assert lay.shade_bytes == 64 * s.n_tri
    assert lay.node_bytes % 64 == 0 and 0 < lay.node_bytes < 64 * len(nodes)
    assert lay.device_bytes == (lay.node_bytes + lay.stream_bytes + lay.shade_bytes
                                + (MATERIAL.itemsize + 8) * len(s.mats) + 16 * QUAD_LIGHT.itemsize)
    assert lay.depth > 0
    # tree modes differ in their nodes, not in the triangle data
    ref = layout(s.tris, len(s.mats), nodes, 0)
    assert ref.digest != lay.digest and ref.stream_bytes == lay.stream_bytes


def test_layout_is_deterministic_on_a_small_scene():
    s = scenes.c0(16, 16)
    a = layout(s.tris, len(s.mats), s.nodes)
    b = layout(s.tris.copy(), len(s.mats), s.nodes.copy())
    assert a.digest == b.digest
    t = s.tris.copy()
    t["v1"][0, 0] += np.float32(1e-3)                      # one vertex moved: another stream
    nodes = scenes.refit_bvh(t, s.nodes)
    assert layout(t, len(s.mats), nodes).digest != a.digest


def test_layout_refuses_what_the_upload_refuses():
    s = scenes.c1(16, 16, level=3)
    L = N.lib()
    out = N.SceneLayout()

    def call(tris, n_mat, nodes, tree=1):
        return L.yc_scene_layout(ptr(tris), len(tris), n_mat, ptr(nodes), len(nodes), tree, C.byref(out))
    assert call(s.tris, len(s.mats), s.nodes) == 0
    assert call(s.tris, len(s.mats), s.nodes, tree=3) == -1
    assert call(s.tris, 1, s.nodes) == -1                  # matID beyond the materials
    assert b"matID" in L.yc_last_error()
    bad = s.nodes.copy()
    k = int(np.nonzero((bad["vert_len"] <= 0) & (bad["child_idx"] > 0))[0][0])
    bad["child_idx"][k] = len(bad) + 5                      # children outside the array
    assert call(s.tris, len(s.mats), bad) == -1
    assert L.yc_last_error()
    bad = s.nodes.copy()
    j = int(np.nonzero(bad["vert_len"] > 0)[0][0])
    bad["vert_list"][j, 0] = len(s.tris)                    # a triangle that does not exist
    assert call(s.tris, len(s.mats), bad) == -1
    assert L.yc_scene_layout(None, 0, 0, None, 0, 1, None) == -1


@pytest.mark.parametrize("kind,n", [("coincident", 3000), ("grid", 140000), ("random", 140000)])
def test_sah_over_leaves_independent_of_host_threads(kind, n):
    """The SAH build over the reference leaves (tree mode 1) chooses the same splits whatever
    the host threads: leaf boxes that all coincide (every split halves the list), boxes on an
    integer grid with zeros of both signs (equal costs; -0 and +0 met in one min or max in
    different orders by different chunkings) and random boxes; ranges above 64K leaves are
    reduced in chunks on threads."""
    s = leafgen.leaf_scene(n, kind, seed=3)
    L = N.lib()
    got = {}
    try:
        for th in (1, 3, 0):
            assert L.yh_set_host_threads(th) == 0
            lay = scenes.layout(s, 1)
            got[th] = (lay["digest"], lay["depth"], lay["node_bytes"])
    finally:
        L.yh_set_host_threads(0)
    assert len(set(got.values())) == 1, got
    assert got[0][2] == 64 * (n - 1)
    if kind == "coincident":   # halving: a balanced tree
        assert got[0][1] == int(np.ceil(np.log2(n))) + 1


def test_first_bad_material_is_named(big):
    """The material check runs on the host's threads and still names the first triangle
    whose matID is out of range, whatever the thread count."""
    s, nodes = big
    t = s.tris.copy()
    t["matID"][200_000] = len(s.mats)
    t["matID"][70_001] = -1
    L = N.lib()
    try:
        for th in (1, 3, 0):
            assert L.yh_set_host_threads(th) == 0
            out = N.SceneLayout()
            assert L.yc_scene_layout(ptr(t), len(t), len(s.mats), ptr(nodes), len(nodes), 1, C.byref(out)) == -1
            assert b"triangle 70001 " in L.yc_last_error()
    finally:
        L.yh_set_host_threads(0)
