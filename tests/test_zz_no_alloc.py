"""yc_render_pass_noalloc: the tile render that allocates no device memory, for callers
that cannot call cudaMalloc while they render (a real-time frame loop that must not take
cudaMalloc's implicit synchronisation, or a host whose device memory is owned by its
own allocator). Its wavefront state lives in a static device array of the library, so
it must give the same accumulator as yc_render_pass for the same tile, call after call,
and must not allocate.

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


def _noalloc(r, sid, aid, seed, reset, cfg):
    c = cfg_struct(cfg)
    N.check(N.lib().yc_render_pass_noalloc(r.h, sid, aid, int(seed) & 0xFFFFFFFF, reset, 1, C.byref(c)), "noalloc")


def _free_device_bytes():
    import torch
    return torch.cuda.mem_get_info(0)[0]


# (scene, frame, options): the default configuration, then options the tile render must
# pass through as yc_render_pass does (Lambert, no MIS, a short GI loop, the reference's
# roulette depth) and a scene with a dielectric sphere
CASES = [
    ("c0", lambda: scenes.c0(96, 80), {}),
    ("c0_lambert_nomis", lambda: scenes.c0(96, 80), dict(brdf_model=0, mis=0, rr_threshold=6, max_depth=4)),
    ("c1_glass", lambda: scenes.c1(96, 80, level=3), dict(max_depth=16, mis_lobe_fix=0)),
]


@pytest.mark.parametrize("name,make,opts", CASES, ids=[c[0] for c in CASES])
def test_noalloc_tile_matches_render_pass_two_calls_in_a_row(name, make, opts):
    s = make()
    cfg = dict(s.cfg, block=3, block_x=2, block_y=2, **opts)     # 48 x 40 tile, the bottom-right block
    seeds = scenes.pass_seeds(31, 2)
    with Renderer(0) as r:
        sid = r.upload(s)
        r.set_camera(s.cam)
        a_ref = r.alloc_accum(96, 80)
        a_na = r.alloc_accum(96, 80)
        for k, sd in enumerate(seeds):
            reset = 1 if k == 0 else 0
            r.render(sid, a_ref, int(sd), reset=reset, cfg=cfg)
            _noalloc(r, sid, a_na, sd, reset, cfg)
            got, want = r.read_accum(a_na), r.read_accum(a_ref)
            assert np.array_equal(got.view(np.int32), want.view(np.int32)), "call %d differs from yc_render_pass" % k
            # only the tile was written
            assert np.all(got[:40, :, 3] == 0) and np.all(got[:, :48, 3] == 0)
            assert np.all(got[40:, 48:, 3] == k + 1)


def test_noalloc_calls_allocate_nothing():
    """After the scene, the accumulators and one warm-up call exist, further calls -- on
    another tile, into another accumulator, with other options -- leave the library's
    device-allocation count and the device's free memory unchanged."""
    s = scenes.c1(128, 128, level=3)
    with Renderer(0) as r:
        sid = r.upload(s)
        r.set_camera(s.cam)
        a1 = r.alloc_accum(128, 128)
        a2 = r.alloc_accum(128, 128)
        _noalloc(r, sid, a1, 7, 1, dict(s.cfg, block=0, block_x=2, block_y=2))
        n0, free0 = N.device_allocations(), _free_device_bytes()
        for k in range(4):
            _noalloc(r, sid, a1, 8 + k, 0, dict(s.cfg, block=k, block_x=2, block_y=2))
            _noalloc(r, sid, a2, 20 + k, 1, dict(s.cfg, block=k, block_x=2, block_y=2, max_depth=3))
        assert N.device_allocations() == n0
        assert _free_device_bytes() == free0
        # the whole frame was covered: every pixel of a2 holds one pass
        assert np.all(r.read_accum(a2)[..., 3] == 1)


def test_noalloc_rejects_tiles_beyond_its_scratch():
    s = scenes.c0(256, 128)       # 32768 pixels in one tile > 16384
    with Renderer(0) as r:
        sid = r.upload(s)
        r.set_camera(s.cam)
        aid = r.alloc_accum(256, 128)
        c = cfg_struct(s.cfg)
        rc = N.lib().yc_render_pass_noalloc(r.h, sid, aid, 1, 1, 1, C.byref(c))
        assert rc == N.YC_E_INVALID
        assert b"16384" in N.lib().yc_last_error()
        # split into 2 x 1 blocks of 16384 pixels it is accepted
        c2 = cfg_struct(dict(s.cfg, block=1, block_x=2, block_y=1))
        N.check(N.lib().yc_render_pass_noalloc(r.h, sid, aid, 1, 1, 1, C.byref(c2)), "noalloc")
