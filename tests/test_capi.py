"""The C-ABI library: it loads, exports every function include/*.h declares, and
rejects bad arguments without touching a GPU."""
import ctypes as C
import os
import re

import numpy as np

from yune_gb300 import _native as N
from yune_gb300.layouts import BVH_NODE, CAM, MATERIAL, QUAD_LIGHT, TRIANGLE

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = []
    for h in ("yune_cuda.h", "yune_host.h"):
        with open(os.path.join(ROOT, "include", h)) as f:
            txt = f.read()
        names += re.findall(r"^(?:int|void|const char\*)\s+(y[ch]_\w+)\s*\(", txt, flags=re.M)
    return sorted(set(names))


def test_exports_every_declared_symbol():
    L = N.lib()
    names = _declared()
    assert len(names) > 30
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    # and the bindings cover them all
    assert not [n for n in names if n not in N.SIGNATURES]


def test_layout_sizes_match_headers():
    assert TRIANGLE.itemsize == 112 and BVH_NODE.itemsize == 80 and MATERIAL.itemsize == 80
    assert CAM.itemsize == 80 and QUAD_LIGHT.itemsize == 128


def test_argument_errors_without_gpu():
    L = N.lib()
    assert L.yc_create(0, None) == -1            # YC_E_INVALID
    assert L.yc_upload_scene(None, None, 0, None, 0, None, 0, None, 0, None) == -1
    assert b"NULL" in L.yc_last_error()
    assert L.yc_render_pass(None, 1, 1, 0, 1, 1, None) == -1
    assert L.yc_destroy(None) == 0
    h = C.c_void_p()
    rc = L.yc_create(0, C.byref(h))
    if rc != 0:   # a machine without a GPU reports no device, it does not crash
        assert rc in (-5, -3)
        assert L.yc_last_error()
    else:
        L.yc_destroy(h)


def test_host_producer_errors():
    L = N.lib()
    h = C.c_void_p()
    assert L.yh_bvh_build(None, 5, 20, 10, C.byref(h)) == -1
    t = np.zeros(1, TRIANGLE)
    assert L.yh_bvh_build(t.ctypes.data, 1, 20, 11, C.byref(h)) == -1   # leaf > 10
    assert L.yh_set_host_threads(-1) == -1 and L.yh_get_host_threads() >= 1
    from yune_gb300 import scenes
    try:
        assert scenes.set_host_threads(3) == 3
    finally:
        assert scenes.set_host_threads(0) >= 1
    assert L.yh_scene_add_icosphere(None, None, 1.0, 2, 0.0, 0, 0) == -1
