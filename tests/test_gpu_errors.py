"""Failures a render call reports to its caller instead of returning wrong pixels, as the
reference surfaces every failed OpenCL call (CLManager::checkError,
src/CLManager.cpp:755-855). Every case is made on the host with a bound the caller sets
(YC_OPT_STACK_LIMIT, YC_OPT_MAX_ROUNDS, the batch's stack_cap); no kernel faults, and
the context stays usable: a normal pass afterwards equals the oracle.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle_py as O
from yune_gb300 import _native as N
from yune_gb300 import scenes
from yune_gb300.batch import Batch
from yune_gb300.core import Renderer, cfg_struct

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def glass():
    return scenes.c1(32, 24, level=4)


def _clean_pass_equals_oracle(r, s, sid):
    seeds = scenes.pass_seeds(5, 1)
    aid = r.alloc_accum(s.width, s.height)
    r.render_passes(sid, aid, seeds, reset_first=1, cfg=s.cfg)
    gpu = r.read_accum(aid)
    r.free_accum(aid)
    ref = np.zeros((s.height, s.width, 4), np.float32)
    O.render(s, ref, seeds[0], 1, s.cfg)
    assert np.array_equal(gpu.view(np.int32), ref.view(np.int32))


def test_stack_limit_overflow_is_an_error(glass):
    s = glass
    with Renderer(0) as r:
        sid = r.upload(s)
        r.set_camera(s.cam)
        depth = r.scene_depth(sid)
        assert depth >= 4
        aid = r.alloc_accum(s.width, s.height)
        r.set_stack_limit(3)   # one level of the hierarchy pushed at most
        with pytest.raises(N.YuneError) as e:
            r.render(sid, aid, 1, reset=1, cfg=s.cfg)
        assert e.value.code == N.YC_E_OVERFLOW
        assert "stack" in str(e.value)
        # the same bound through the allocation-free tile render
        c = cfg_struct(s.cfg)
        assert N.lib().yc_render_pass_noalloc(r.h, sid, aid, 1, 1, 1, C.byref(c)) == N.YC_E_OVERFLOW
        # a bound the scene fits in is no error
        r.set_stack_limit(depth + 2)
        r.render(sid, aid, 1, reset=1, cfg=s.cfg)
        r.set_stack_limit(0)
        r.free_accum(aid)
        _clean_pass_equals_oracle(r, s, sid)


def test_round_bound_is_a_timeout(glass):
    s = glass
    with Renderer(0) as r:
        sid = r.upload(s)
        r.set_camera(s.cam)
        aid = r.alloc_accum(s.width, s.height)
        # one trace + shade round, and no tail kernel (which finishes a frame this small
        # inside that round): every path that bounces is still live
        r.set_tail_paths(0)
        r.set_max_rounds(1)
        with pytest.raises(N.YuneError) as e:
            r.render(sid, aid, 1, reset=1, cfg=s.cfg)
        assert e.value.code == N.YC_E_TIMEOUT
        assert "rounds" in str(e.value)
        c = cfg_struct(s.cfg)
        assert N.lib().yc_render_pass_noalloc(r.h, sid, aid, 1, 1, 1, C.byref(c)) == N.YC_E_TIMEOUT
        r.set_max_rounds(1000000)
        r.set_tail_paths(-1)
        r.free_accum(aid)
        _clean_pass_equals_oracle(r, s, sid)


def test_batch_stack_cap_overflow_is_an_error(glass):
    s = glass
    with Renderer(0) as r:
        sid = r.upload(s)
        aid = r.alloc_accum(s.width, s.height)
        b = Batch(r, pool_paths=1 << 14, rounds_per_launch=4, stack_cap=3, sort_threshold=0)
        b.add_job(sid, aid, s.cam, scenes.pass_seeds(3, 2), s.cfg)
        with pytest.raises(N.YuneError) as e:
            b.run()
        assert e.value.code == N.YC_E_OVERFLOW
        b.close()
        r.set_camera(s.cam)
        r.free_accum(aid)
        _clean_pass_equals_oracle(r, s, sid)
