"""The bidirectional tracer with multiple importance sampling (YC_BDPT_MIS) on the GPU,
called through the C-ABI.

Parity: against its CPU statement (oracle/bdpt_mis_oracle.hpp) at equal seeds, every
pixel within 1e-3 relative (the arithmetic is the same, so the expectation is equal bits)
and the ray counts per kind equal. Convergence: against an independent estimator of the
same image, the next-event-only unidirectional tracer run to 65,536 FP64 passes
(tests/golden/fp64_c0_mis.npz, fp64_c0_bdpt_mis.npz): the mean error over the 1,024
reference pixels stays within 5 standard errors, and the error trimmed of the 1% worst
pixels halves when the passes quadruple."""
import numpy as np
import pytest

from oracle import oracle_py as O
from yune_gb300 import quality, scenes
from yune_gb300.core import Renderer

pytestmark = pytest.mark.gpu

REL_TOL = 1e-3


@pytest.fixture(scope="module")
def renderer():
    with Renderer(0) as r:
        yield r


def _rel_bad(gpu, ref):
    a, b = gpu[..., :3].astype(np.float64), ref[..., :3].astype(np.float64)
    both_nan = np.isnan(a) & np.isnan(b)
    rel = np.abs(a - b) / np.maximum(np.abs(b), 1e-6)
    return int((~((rel <= REL_TOL) | both_nan)).any(axis=-1).sum())


def _scene(name, w, h, kmax):
    if name == "c0_mis":
        return scenes.c0_mis(w, h, kmax=kmax)
    return scenes.c0_bdpt_mis(w, h, bounces=kmax, lights=4 if name == "c0_bdpt_mis" else 1)


def _render_gpu(r, s, seeds, shade_sort=None):
    sid = r.upload(s)
    r.set_camera(s.cam)
    if shade_sort is not None:
        r.set_shade_sort(shade_sort)
    aid = r.alloc_accum(s.width, s.height)
    r.reset_stats()
    r.render_passes(sid, aid, seeds, reset_first=1, cfg=s.cfg)
    img = r.read_accum(aid)
    st = r.stats()
    if shade_sort is not None:
        r.set_shade_sort(65536)
    r.free_accum(aid)
    r.release(sid)
    return img, st


def _render_oracle(s, seeds, kmax, heap_size=1500):
    ref = np.zeros((s.height, s.width, 4), np.float32)
    tot = {}
    for k, sd in enumerate(seeds):
        c = O.render_bdpt_mis(s, ref, sd, 1 if k == 0 else 0, kmax, s.cfg, heap_size=heap_size)
        assert c["heap_overflow"] == 0
        for key, v in c.items():
            tot[key] = tot.get(key, 0) + v
    return ref, tot


@pytest.mark.parametrize("name,kmax", [("c0_mis", 20), ("c0_bdpt_mis", 8), ("c0_bdpt_mis", 3), ("c0_bdpt_mis1", 5)])
def test_render_parity_bdpt_mis(renderer, name, kmax):
    s = _scene(name, 40, 32, kmax)
    seeds = scenes.pass_seeds(8, 2)
    gpu, st = _render_gpu(renderer, s, seeds)
    ref, cnt = _render_oracle(s, seeds, kmax)
    assert st["stack_overflow"] == 0
    assert _rel_bad(gpu, ref) == 0
    assert np.array_equal(gpu[..., 3], ref[..., 3])
    assert st["samples"] == 40 * 32 * 2
    assert (st["primary"], st["extension"], st["shadow"], st["connection"]) == \
        (cnt["primary"], cnt["extension"], cnt["shadow"], cnt["mis"])
    assert st["rays"] == cnt["rays"]


def test_bdpt_mis_shade_sort_gives_the_same_pass(renderer):
    """Every round's shade queue sorted by path state and material class (a frame large
    enough to be sorted): every pixel against the oracle, the ray count unchanged."""
    s = scenes.c0_bdpt_mis(1024, 512)
    seeds = scenes.pass_seeds(13, 1)
    renderer.set_profiling(True)
    gpu, st = _render_gpu(renderer, s, seeds, shade_sort=1)
    kt = renderer.kernel_times()
    renderer.set_profiling(False)
    assert kt["sort_launches"] > 0
    ref, cnt = _render_oracle(s, seeds, 8)
    assert _rel_bad(gpu, ref) == 0
    assert np.array_equal(gpu[..., 3], ref[..., 3])
    assert st["rays"] == cnt["rays"]


@pytest.mark.parametrize("name,passes", [("c0_mis", 16), ("c0_bdpt_mis", 16)])
def test_bdpt_mis_converges_to_the_unidirectional_image(renderer, name, passes):
    s = scenes.CONFIGS[name]()
    ref = quality.load_reference(name)
    assert ref is not None and ref["n_pass"] == 65536
    seeds = scenes.pass_seeds(5, 4 * passes)
    sid = renderer.upload(s)
    renderer.set_camera(s.cam)
    aid = renderer.alloc_accum(s.width, s.height)
    renderer.render_passes(sid, aid, seeds[:passes], reset_first=1, cfg=s.cfg)
    trim1 = quality.trimmed_rmse(renderer.read_accum(aid), ref)
    renderer.render_passes(sid, aid, seeds[passes:], reset_first=0, cfg=s.cfg)
    img = renderer.read_accum(aid)
    renderer.free_accum(aid)
    renderer.release(sid)
    rmse4, rel4, bias4 = quality.error(img, ref)
    trim4 = quality.trimmed_rmse(img, ref)
    assert np.all(img[..., 3] == 4 * passes)
    assert abs(bias4) < 5.0 * rmse4 / np.sqrt(len(ref["xs"]))
    assert 1.5 < trim1 / trim4 < 2.7   # 1/sqrt(passes): 2 expected
