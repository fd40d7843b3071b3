"""The binary scene cache (yh_cache_save / yh_cache_query / yh_cache_load): a scene read
back is byte-identical to the one written, and every damaged, foreign or stale file is
refused with its status code instead of being read as a scene. CPU only."""
import ctypes as C
import os

import numpy as np
import pytest

from yune_gb300 import _native as N
from yune_gb300 import scenes
from yune_gb300.layouts import BVH_NODE, CAM, MATERIAL, QUAD_LIGHT, TRIANGLE

FIELDS = ("tris", "mats", "lights", "nodes", "cam")


def _same(a, b):
    for f in FIELDS:
        x, y = getattr(a, f), getattr(b, f)
        assert x.dtype == y.dtype and x.shape == y.shape, f
        assert x.tobytes() == y.tobytes(), f
    assert a.depth == b.depth and a.width == b.width and a.height == b.height and a.spp == b.spp
    assert a.cfg == b.cfg and a.name == b.name


@pytest.fixture(scope="module")
def glass():
    # 81,954 triangles: the triangle and node sections span several 4 MiB hash chunks
    return scenes.c1(64, 48, level=6)


def test_round_trip_is_byte_identical(tmp_path, glass):
    p = str(tmp_path / "c1.ysc")
    key = scenes.cache_key("c1", width=64, height=48, level=6)
    scenes.save_cache(glass, p, key)
    _same(glass, scenes.load_cache(p, key))
    info = N.CacheInfo()
    assert N.lib().yh_cache_query(os.fsencode(p), C.byref(info)) == 0
    assert (info.key, info.n_tri, info.n_node, info.has_cam) == (key, glass.n_tri, len(glass.nodes), 1)


def test_file_layout(tmp_path):
    """Header fields and 64-byte aligned sections where the header comment puts them."""
    s = scenes.c0(16, 16)
    p = str(tmp_path / "c0.ysc")
    scenes.save_cache(s, p, 7)
    raw = open(p, "rb").read()
    assert raw[:8] == b"YUNESCEN"
    u32 = np.frombuffer(raw[8:40], "<u4")
    assert u32[0] == 1 and u32[1] == 0x01020304
    assert list(u32[2:7]) == [TRIANGLE.itemsize, MATERIAL.itemsize, QUAD_LIGHT.itemsize, BVH_NODE.itemsize,
                              CAM.itemsize]
    u64 = np.frombuffer(raw[40:160], "<u8")
    key, count, offset, size = u64[0], u64[1:7], u64[7:13], u64[13]
    assert key == 7 and size == len(raw) and size % 64 == 0
    assert list(count[:5]) == [s.n_tri, len(s.mats), len(s.lights), len(s.nodes), 1]
    assert all(o % 64 == 0 for o in offset) and offset[0] == 256
    tri = np.frombuffer(raw, TRIANGLE, count=s.n_tri, offset=int(offset[0]))
    assert tri.tobytes() == s.tris.tobytes()


def test_stale_key_is_refused(tmp_path):
    s = scenes.c0(16, 16)
    p = str(tmp_path / "c0.ysc")
    scenes.save_cache(s, p, 11)
    with pytest.raises(N.YuneError) as e:
        scenes.load_cache(p, 12)
    assert e.value.code == N.YH_E_STALE
    # the C entry point checks the key itself, not only the Python wrapper
    tris = np.empty(s.n_tri, TRIANGLE)
    rc = N.lib().yh_cache_load(os.fsencode(p), 12, tris.ctypes.data, len(tris), None, 0, None, 0, None, 0, None,
                               None, 0)
    assert rc == N.YH_E_STALE


def _damaged(tmp_path, glass, edit):
    p = str(tmp_path / "d.ysc")
    scenes.save_cache(glass, p, 5)
    raw = bytearray(open(p, "rb").read())
    raw = edit(raw)
    with open(p, "wb") as f:
        f.write(raw)
    return p


@pytest.mark.parametrize("where", ["header", "triangles", "last node", "camera", "caller bytes"])
def test_flipped_byte_is_refused(tmp_path, glass, where):
    def flip(raw):
        u64 = np.frombuffer(bytes(raw[40:160]), "<u8")
        count, offset = u64[1:7], u64[7:13]
        pos = {"header": 20, "triangles": int(offset[0]) + 5 * 1024 * 1024 + 3,
               "last node": int(offset[3] + count[3] * BVH_NODE.itemsize) - 7, "camera": int(offset[4]) + 12,
               "caller bytes": int(offset[5]) + 2}[where]
        raw[pos] ^= 0x10
        return raw
    p = _damaged(tmp_path, glass, flip)
    with pytest.raises(N.YuneError) as e:
        scenes.load_cache(p, 5)
    assert e.value.code == N.YH_E_FORMAT


@pytest.mark.parametrize("cut", [0, 100, 256, 4096, -64, -1])
def test_truncated_or_extended_file_is_refused(tmp_path, glass, cut):
    def trim(raw):
        return raw[:cut] if cut > 0 else (raw[:len(raw) + cut] if cut < 0 else raw + b"\0" * 64)
    p = _damaged(tmp_path, glass, trim)
    with pytest.raises(N.YuneError) as e:
        scenes.load_cache(p, 5)
    assert e.value.code == N.YH_E_FORMAT


def test_foreign_and_missing_files(tmp_path):
    p = str(tmp_path / "not_a_cache.bin")
    with open(p, "wb") as f:
        f.write(np.random.default_rng(3).bytes(4096))
    with pytest.raises(N.YuneError) as e:
        scenes.load_cache(p, 0)
    assert e.value.code == N.YH_E_FORMAT
    with pytest.raises(N.YuneError) as e:
        scenes.load_cache(str(tmp_path / "absent.ysc"), 0)
    assert e.value.code == N.YH_E_IO
    s = scenes.c0(16, 16)
    with pytest.raises(N.YuneError) as e:
        scenes.save_cache(s, str(tmp_path / "no_such_dir" / "x.ysc"), 0)
    assert e.value.code == N.YH_E_IO


def test_capacities_and_arguments(tmp_path):
    s = scenes.c0(16, 16)
    p = str(tmp_path / "c0.ysc")
    scenes.save_cache(s, p, 9)
    L = N.lib()
    bp = os.fsencode(p)
    tris = np.empty(s.n_tri, TRIANGLE)
    mats = np.empty(len(s.mats), MATERIAL)
    lights = np.empty(len(s.lights), QUAD_LIGHT)
    nodes = np.empty(len(s.nodes), BVH_NODE)
    cam = np.empty(1, CAM)
    meta = C.create_string_buffer(4096)

    def load(n_tri=s.n_tri, cam_ptr=cam.ctypes.data, tri_ptr=tris.ctypes.data):
        return L.yh_cache_load(bp, 9, tri_ptr, n_tri, mats.ctypes.data, len(mats), lights.ctypes.data,
                               len(lights), nodes.ctypes.data, len(nodes), cam_ptr, meta, 4096)
    assert load() == 0
    assert load(n_tri=s.n_tri - 1) == N.YH_E_RANGE      # too little room
    assert load(cam_ptr=None) == N.YH_E_RANGE           # the file has a camera
    assert load(tri_ptr=None) == N.YH_E_INVALID         # room claimed, no array
    assert L.yh_cache_save(bp, 0, None, 3, None, 0, None, 0, None, 0, -1, None, None, 0) == N.YH_E_INVALID
    assert L.yh_cache_save(None, 0, None, 0, None, 0, None, 0, None, 0, -1, None, None, 0) == N.YH_E_INVALID
    assert L.yh_cache_query(bp, None) == N.YH_E_INVALID


def test_empty_scene_without_camera(tmp_path):
    p = os.fsencode(str(tmp_path / "empty.ysc"))
    L = N.lib()
    assert L.yh_cache_save(p, 3, None, 0, None, 0, None, 0, None, 0, -1, None, None, 0) == 0
    info = N.CacheInfo()
    assert L.yh_cache_query(p, C.byref(info)) == 0
    assert (info.n_tri, info.n_mat, info.n_light, info.n_node, info.has_cam, info.meta_bytes, info.depth) == \
        (0, 0, 0, 0, 0, 0, -1)
    assert L.yh_cache_load(p, 3, None, 0, None, 0, None, 0, None, 0, None, None, 0) == 0


def test_cached_builds_once_then_reads(tmp_path, monkeypatch):
    p = str(tmp_path / "c0.ysc")
    a = scenes.cached("c0", p, width=32, height=24)
    assert os.path.exists(p)
    calls = []
    real = scenes.CONFIGS["c0"]
    monkeypatch.setitem(scenes.CONFIGS, "c0", lambda **kw: calls.append(kw) or real(**kw))
    b = scenes.cached("c0", p, width=32, height=24)
    assert calls == []                                  # read back, not rebuilt
    _same(a, b)
    c = scenes.cached("c0", p, width=32, height=24, seed=4)   # other parameters: rebuilt and rewritten
    assert calls == [dict(width=32, height=24, seed=4)]
    assert c.tris.tobytes() != a.tris.tobytes()
    _same(c, scenes.load_cache(p, scenes.cache_key("c0", width=32, height=24, seed=4)))


def test_concurrent_writers_leave_one_whole_file(tmp_path):
    """Writers of one path in parallel: each writes its own temporary file and renames it
    into place, so the file read afterwards is one writer's scene, whole."""
    import threading
    p = str(tmp_path / "shared.ysc")
    made = {k: scenes.c0(16, 16, seed=k) for k in range(1, 5)}
    threads = [threading.Thread(target=scenes.save_cache, args=(s, p, k)) for k, s in made.items()]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    info = N.CacheInfo()
    assert N.lib().yh_cache_query(os.fsencode(p), C.byref(info)) == 0
    _same(made[info.key], scenes.load_cache(p, info.key))
    assert sorted(os.listdir(tmp_path)) == ["shared.ysc"]   # no temporary file left behind
