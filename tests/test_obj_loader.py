"""OBJ/MTL ingestion (yh_scene_load_obj) against Yune's own loader, Scene::loadModel
(src/Scene.cpp:133-383): the triangle, material and BVH node arrays of the reference,
recorded in tests/golden/obj_*.npz by tests/golden/make_golden.py, and, where the
compiled reference is at hand, compared live."""
import importlib.util
import os

import numpy as np
import pytest

from oracle import build_oracle
from oracle import oracle_py as O
from yune_gb300 import _native as N
from yune_gb300 import scenes

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _module(name):
    spec = importlib.util.spec_from_file_location(name, os.path.join(GOLD, name + ".py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


MG = _module("make_golden")
OBJ = _module("obj_files")
_TREE = build_oracle.reference_tree()
CORNELL = os.path.join(_TREE, "geometry", "cornellbox.obj") if _TREE else None


def _ours(path):
    s = scenes.from_obj(path)
    return s.tris, s.mats, s.nodes


def _check(got, want):
    for k in want.files if hasattr(want, "files") else want:
        a, b = np.asarray(got[k]), np.asarray(want[k])
        assert a.shape == b.shape, k
        assert np.array_equal(a.view(np.uint8), b.view(np.uint8)), k


def test_test_scene_by_hand(tmp_path):
    """The rules read off Scene::loadModel, on a file written for the test."""
    tris, mats, _ = _ours(OBJ.write(str(tmp_path)))
    assert len(tris) == 5 and len(mats) == 2
    assert list(tris["matID"]) == [0, 0, 0, 0, 1]   # unknown name and the second object: 0
    assert np.array_equal(tris["v3"][2], [1, -1, 1, 1])   # a quad gives its first three vertices
    assert np.array_equal(tris["vn1"][2], [0, 1, 0, 0])   # v/vt/vn: the normal index
    assert np.array_equal(tris["vn2"][3], [0, 0, 0, 0])   # no normal indices: zeros
    white, glass = mats[0], mats[1]
    assert np.allclose(white["kd"], [0.8, 0.8, 0.8, 1]) and np.array_equal(white["ks"], [0, 0, 0, 1])
    assert white["px"] == 1 and white["alpha_x"] == 100   # defaults of newMaterial
    assert glass["px"] == 3 and glass["py"] == 7           # px and py swapped
    assert glass["n"] == np.float32(1.5) and glass["alpha_x"] == np.float32(0.25)
    assert glass["is_specular"] == 1 and glass["is_transmissive"] == 1


def test_test_scene_matches_reference_loader(tmp_path):
    got = MG.obj_fields(*_ours(OBJ.write(str(tmp_path))))
    _check(got, np.load(os.path.join(GOLD, "obj_test_scene.npz")))


def test_cornellbox_matches_reference_loader():
    if not CORNELL or not os.path.exists(CORNELL):
        pytest.skip("the reference's Cornell-box OBJ is not on this machine")
    got = MG.obj_fields(*_ours(CORNELL))
    _check(got, np.load(os.path.join(GOLD, "obj_cornellbox.npz")))


def test_live_against_the_compiled_reference(tmp_path):
    L = O.ref()
    if L is None or not hasattr(L, "ref_load_obj"):
        pytest.skip("compiled reference loader not built here")
    path = OBJ.write(str(tmp_path))
    want = MG.obj_fields(*O.ref_load_obj(path), no_normals=OBJ.NO_NORMALS)
    _check(MG.obj_fields(*_ours(path)), want)
    if CORNELL and os.path.exists(CORNELL):
        _check(MG.obj_fields(*_ours(CORNELL)), MG.obj_fields(*O.ref_load_obj(CORNELL)))


def test_errors(tmp_path):
    b = scenes.Builder()
    with pytest.raises(N.YuneError) as e:
        b.load_obj(str(tmp_path / "missing.obj"))
    assert e.value.code == -1
    bad = tmp_path / "bad.obj"
    bad.write_text("v 0 0 0\nv 1 0 0\nf 1 2 3\n")
    with pytest.raises(N.YuneError) as e:
        scenes.Builder().load_obj(str(bad))
    assert e.value.code == -3   # index 3 is beyond the two vertices read
    nomtl = tmp_path / "nomtl.obj"
    nomtl.write_text("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n")
    b = scenes.Builder()
    assert b.load_obj(str(nomtl)) == 1
    tris, mats, _ = b.arrays()
    assert len(mats) == 1 and np.allclose(mats[0]["kd"], [0.3, 0.3, 0.3, 1])   # the default material
