"""yc_render_pass_noalloc: the tile render that allocates no device memory, for callers
that cannot call cudaMalloc while they render (a real-time frame loop that must not take
cudaMalloc's implicit synchronisation, or a host whose device memory is owned by its
own allocator). Its wavefront state lives in a static device array of the library, so
it must give the same accumulator as yc_render_pass for the same tile, call after call.

This file is named so pytest collects it last: it passes alone in a fresh process and
after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

from yune_gb300 import _native as N
from yune_gb300 import scenes
from yune_gb300.core import Renderer, cfg_struct

pytestmark = pytest.mark.gpu

REL_TOL = 1e-3   # the per-pixel tolerance of the render parity tests


def _close(a, b):
    x, y = a[..., :3].astype(np.float64), b[..., :3].astype(np.float64)
    rel = np.abs(x - y) / np.maximum(np.abs(y), 1e-6)
    return bool((rel <= REL_TOL).all()) and np.array_equal(a[..., 3], b[..., 3])


def test_noalloc_tile_matches_render_pass_two_calls_in_a_row():
    s = scenes.c0(96, 80)
    cfg = dict(s.cfg, block=3, block_x=2, block_y=2)     # 48 x 40 tile, the bottom-right block
    seeds = scenes.pass_seeds(31, 2)
    with Renderer(0) as r:
        sid = r.upload(s)
        r.set_camera(s.cam)
        a_ref = r.alloc_accum(96, 80)
        a_na = r.alloc_accum(96, 80)
        L = N.lib()
        c = cfg_struct(cfg)
        for k, sd in enumerate(seeds):
            reset = 1 if k == 0 else 0
            r.render(sid, a_ref, int(sd), reset=reset, cfg=cfg)
            N.check(L.yc_render_pass_noalloc(r.h, sid, a_na, int(sd), reset, 1, C.byref(c)), "noalloc")
            got, want = r.read_accum(a_na), r.read_accum(a_ref)
            assert _close(got, want), "call %d differs from yc_render_pass" % k
            # only the tile was written
            assert np.all(got[:40, :, 3] == 0) and np.all(got[:, :48, 3] == 0)
            assert np.all(got[40:, 48:, 3] == k + 1)


def test_noalloc_rejects_tiles_beyond_its_scratch():
    s = scenes.c0(256, 128)       # 32768 pixels in one tile > 16384
    with Renderer(0) as r:
        sid = r.upload(s)
        r.set_camera(s.cam)
        aid = r.alloc_accum(256, 128)
        c = cfg_struct(s.cfg)
        rc = N.lib().yc_render_pass_noalloc(r.h, sid, aid, 1, 1, 1, C.byref(c))
        assert rc == -1
        assert b"16384" in N.lib().yc_last_error()
        # split into 2 x 1 blocks of 16384 pixels it is accepted
        c2 = cfg_struct(dict(s.cfg, block=1, block_x=2, block_y=1))
        N.check(N.lib().yc_render_pass_noalloc(r.h, sid, aid, 1, 1, 1, C.byref(c2)), "noalloc")
