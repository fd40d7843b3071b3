"""BVH::createBVH on the GPU (yc_bvh_build) against the host builder, whose node arrays
equal the reference's (tests/test_oracle_pin.py): every node's box, child index, count and
triangle list, bounds compared as values (a zero bound is stored as +0 on the GPU)."""
import numpy as np
import pytest

from yune_gb300 import scenes, workloads
from yune_gb300.core import Renderer

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def renderer():
    with Renderer(0) as r:
        yield r


def _same(a, b):
    assert len(a) == len(b), (len(a), len(b))
    assert np.array_equal(a["child_idx"], b["child_idx"])
    assert np.array_equal(a["vert_len"], b["vert_len"])
    used = np.arange(10)[None, :] < np.maximum(a["vert_len"], 0)[:, None]
    assert np.array_equal(np.where(used, a["vert_list"], -1), np.where(used, b["vert_list"], -1))
    for k in ("p_min", "p_max"):
        assert np.array_equal(a[k], b[k]), k   # value comparison: -0 == +0


def _obj_scene(tmp_path):
    import importlib.util
    import os
    spec = importlib.util.spec_from_file_location("obj_files", os.path.join(os.path.dirname(__file__), "golden",
                                                                            "obj_files.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return scenes.from_obj(m.write(str(tmp_path))).tris


@pytest.mark.parametrize("case,bins,leaf", [("c0", 20, 10), ("c1l4", 20, 4), ("c1l6", 20, 4), ("c1l4", 2, 4),
                                            ("mixed", 20, 4), ("obj", 20, 10)])
def test_device_build_equals_host_build(renderer, tmp_path, case, bins, leaf):
    if case == "c0":
        tris = scenes.c0(8, 8).tris
    elif case == "c1l4":
        tris = scenes.c1(8, 8, level=4).tris
    elif case == "c1l6":
        tris = scenes.c1(8, 8, level=6).tris
    elif case == "mixed":
        tris = workloads.mixed_scene(150_000, 7, 8, 8, 1).tris
    else:
        tris = _obj_scene(tmp_path)
    want, wd = scenes.build_bvh(tris, bins, leaf)
    got, gd = renderer.build_bvh(tris, bins, leaf)
    _same(got, want)
    assert gd == wd


def test_coincident_centroids_are_refused(renderer):
    """More than leaf_max triangles with one centroid: every split sends them to the same
    child and the reference builder never ends; both builders stop with an error."""
    from yune_gb300 import _native as N
    base = scenes.c0(8, 8).tris
    tris = np.concatenate([base] + [base[:1]] * 4)   # five copies of one triangle, leaf_max 2
    with pytest.raises(N.YuneError):
        scenes.build_bvh(tris, 20, 2)
    with pytest.raises(N.YuneError):
        renderer.build_bvh(tris, 20, 2)


def test_device_built_tree_renders_like_the_host_one(renderer):
    """A scene uploaded with the GPU-built node array renders the same bits."""
    s = scenes.c1(40, 32, level=5)
    nodes, depth = renderer.build_bvh(s.tris, 20, 4)
    seeds = scenes.pass_seeds(3, 2)
    out = []
    for nd, dp in ((s.nodes, s.depth), (nodes, depth)):
        s2 = scenes.SceneData(s.tris, s.mats, s.lights, nd, dp, s.cam, 40, 32, 2, s.cfg, "c1")
        sid = renderer.upload(s2)
        renderer.set_camera(s.cam)
        aid = renderer.alloc_accum(40, 32)
        renderer.render_passes(sid, aid, seeds, reset_first=1, cfg=s.cfg)
        out.append(renderer.read_accum(aid))
        renderer.free_accum(aid)
        renderer.release(sid)
    assert np.array_equal(out[0].view(np.int32), out[1].view(np.int32))
