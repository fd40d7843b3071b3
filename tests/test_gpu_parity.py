"""GPU parity: the CUDA core, called through the C-ABI, against the CPU oracle.

Bars (from the core's contract):
  * closest hit: triangle index and t bit-exact, including the choice between triangles
    at exactly the same t (the reference keeps the first its breadth-first walk meets);
  * any-hit: the occlusion boolean is identical;
  * per-pixel radiance after N passes at equal seeds: within 1e-3 relative (the kernel
    arithmetic is the reference's, so the expectation is bit equality);
  * ray counters equal to the oracle's per kind (same algorithm, same random numbers).
"""
import numpy as np
import pytest

from oracle import oracle_py as O
from yune_gb300 import scenes
from yune_gb300.core import Renderer

pytestmark = pytest.mark.gpu

REL_TOL = 1e-3


@pytest.fixture(scope="module")
def renderer():
    with Renderer(0) as r:
        yield r


def _cmp_closest(gpu, orc):
    gt, gl, gtt = gpu
    ot, ol, ott, ov = orc
    assert ov.sum() == 0, "oracle queue overflow on the test rays"
    same = (gt == ot) & (gl == ol) & (gtt.view(np.int32) == ott.view(np.int32))
    diff = ~same
    # a difference is only allowed between triangles hit at exactly the same t
    tie = diff & (gtt.view(np.int32) == ott.view(np.int32)) & (gt >= 0) & (ot >= 0)
    return int(diff.sum()), int(tie.sum())


@pytest.mark.parametrize("tree", [0, 1, 2])
@pytest.mark.parametrize("cfg_name,level", [("c0", None), ("c1", 6)])
def test_trace_closest_and_any(renderer, cfg_name, level, tree):
    s = scenes.c0(64, 64) if cfg_name == "c0" else scenes.c1(64, 64, level=level)
    renderer.set_tree_mode(tree)
    sid = renderer.upload(s)
    renderer.set_tree_mode(1)
    rays = O.seeded_rays(s, 50000 if cfg_name == "c0" else 20000, seed=11)
    g = renderer.trace(sid, rays, any_hit=False)
    o = O.trace(s, rays, any_hit=False)
    ndiff, ntie = _cmp_closest(g, o)
    assert ndiff == 0, "closest hits differ: %d of %d (%d at equal t)" % (ndiff, len(rays), ntie)
    # shadow rays: finite segments toward random points
    seg = rays.copy()
    seg[:, 8] = np.where(np.isfinite(o[2]), o[2] * 1.001, 0.7).astype(np.float32)
    ga, _, _ = renderer.trace(sid, seg, any_hit=True)
    oa = O.trace(s, seg, any_hit=True)[0] >= 0
    oa_light = O.trace(s, seg, any_hit=True)[1] >= 0
    assert np.array_equal(ga.astype(bool), oa | oa_light)
    renderer.release(sid)


@pytest.mark.parametrize("tree", [0, 1, 2])
def test_trace_axis_aligned_rays(renderer, tree):
    """Rays with zero direction components take the reference's NaN-skipping slab path."""
    s = scenes.c0(64, 64)
    renderer.set_tree_mode(tree)
    sid = renderer.upload(s)
    renderer.set_tree_mode(1)
    rng = np.random.default_rng(3)
    n = 6000
    r = np.zeros((n, 9), np.float32)
    r[:, 0:3] = rng.uniform(-0.45, 0.45, (n, 3))
    r[:, 3] = 1.0
    axis = rng.integers(0, 3, n)
    sign = rng.choice([-1.0, 1.0], n)
    r[np.arange(n), 4 + axis] = sign
    # some rays start exactly on a wall plane
    r[:200, 0] = -0.5
    r[:, 8] = np.inf
    g = renderer.trace(sid, r)
    o = O.trace(s, r)
    ndiff, ntie = _cmp_closest(g, o)
    assert ndiff == 0, "closest hits differ: %d (%d at equal t)" % (ndiff, ntie)
    renderer.release(sid)


CFGS = {
    "as_shipped": dict(mis=0, rr_threshold=6, max_depth=100000, brdf_model=0, mis_lobe_fix=0),
    "mis_on_fix": dict(mis=1, rr_threshold=3, max_depth=100000, brdf_model=1, mis_lobe_fix=1),
    "mis_ref": dict(mis=1, rr_threshold=3, max_depth=16, brdf_model=0, mis_lobe_fix=0),
}


def _render_both(renderer, s, W, H, seeds, cfg, gi=1):
    sid = renderer.upload(s)
    renderer.set_camera(s.cam)
    aid = renderer.alloc_accum(W, H)
    renderer.reset_stats()
    full = dict(scenes.default_cfg(), **cfg)
    renderer.render_passes(sid, aid, seeds, reset_first=1, gi_check=gi, cfg=full)
    gpu = renderer.read_accum(aid)
    st = renderer.stats()
    renderer.free_accum(aid)
    renderer.release(sid)
    ref = np.zeros((H, W, 4), np.float32)
    cnt = {}
    for k, sd in enumerate(seeds):
        c = O.render(s, ref, sd, 1 if k == 0 else 0, dict(cfg, gi_check=gi))
        for key, v in c.items():
            cnt[key] = cnt.get(key, 0) + v
    return gpu, ref, st, cnt


def _rel_bad(gpu, ref):
    a, b = gpu[..., :3].astype(np.float64), ref[..., :3].astype(np.float64)
    both_nan = np.isnan(a) & np.isnan(b)
    both_inf = np.isinf(a) & np.isinf(b) & (np.sign(a) == np.sign(b))
    rel = np.abs(a - b) / np.maximum(np.abs(b), 1e-6)
    ok = (rel <= REL_TOL) | both_nan | both_inf
    return int((~ok).any(axis=-1).sum())


@pytest.mark.parametrize("cfg_key", sorted(CFGS))
def test_render_parity_c0(renderer, cfg_key):
    s = scenes.c0(48, 40)
    seeds = scenes.pass_seeds(1234, 3)
    gpu, ref, st, cnt = _render_both(renderer, s, 48, 40, seeds, CFGS[cfg_key])
    assert st["stack_overflow"] == 0
    bad = _rel_bad(gpu, ref)
    assert bad == 0, "%d pixels beyond %g relative" % (bad, REL_TOL)
    assert np.array_equal(gpu[..., 3], ref[..., 3])
    assert st["rays"] == cnt["rays"]
    assert st["shadow"] == cnt["shadow"] and st["mis"] == cnt["mis"] and st["extension"] == cnt["extension"]
    assert st["samples"] == 48 * 40 * 3


def _diff_report(gpu, ref):
    d = np.argwhere(gpu.view(np.int32) != ref.view(np.int32))
    pix = sorted({(int(y), int(x)) for y, x, _ in d})
    return "%d pixels differ, first %s: gpu %s ref %s" % (
        len(pix), pix[:4], [gpu[y, x].tolist() for y, x in pix[:2]], [ref[y, x].tolist() for y, x in pix[:2]])


def test_render_parity_c1_glass(renderer):
    """The benchmark's glass scene (level-6 icosphere, IOR 1.5, NEE + MIS, Oren-Nayar,
    roulette after bounce 3, at most 16 bounces): every pixel bit-equal to the oracle and
    every ray counter equal, as on every other scene."""
    s = scenes.c1(40, 40, level=6)
    seeds = scenes.pass_seeds(99, 2)
    cfg = dict(mis=1, rr_threshold=3, max_depth=16, brdf_model=1, mis_lobe_fix=1)
    gpu, ref, st, cnt = _render_both(renderer, s, 40, 40, seeds, cfg)
    assert cnt["heap_overflow"] == 0
    assert st["stack_overflow"] == 0
    assert np.array_equal(gpu.view(np.int32), ref.view(np.int32)), _diff_report(gpu, ref)
    for key in ("rays", "shadow", "mis", "extension"):
        assert st[key] == cnt[key], (key, st[key], cnt[key])


@pytest.mark.parametrize("mis", [0, 1])
def test_render_parity_udpt_four_lights(renderer, mis):
    """The unidirectional tracer with four quad lights: sampleLights' CDF over the
    lights' weights (udpt.cl:632-698) picks the light of every next-event sample, and
    every pixel and ray counter equals the oracle's."""
    s = scenes.c0_bdpt(40, 32, bounces=8, lights=4)
    assert len(s.lights) == 4
    seeds = scenes.pass_seeds(77, 3)
    cfg = dict(mis=mis, rr_threshold=3, max_depth=16, brdf_model=1, mis_lobe_fix=1)
    gpu, ref, st, cnt = _render_both(renderer, s, 40, 32, seeds, cfg)
    assert cnt["heap_overflow"] == 0
    assert st["stack_overflow"] == 0
    assert np.array_equal(gpu.view(np.int32), ref.view(np.int32)), _diff_report(gpu, ref)
    for key in ("rays", "shadow", "mis", "extension"):
        assert st[key] == cnt[key], (key, st[key], cnt[key])


def test_render_gi_off(renderer):
    s = scenes.c0(32, 32)
    seeds = scenes.pass_seeds(5, 2)
    gpu, ref, st, cnt = _render_both(renderer, s, 32, 32, seeds, CFGS["as_shipped"], gi=0)
    assert _rel_bad(gpu, ref) == 0
    assert st["extension"] == 0


def test_tonemap_parity(renderer):
    s = scenes.c0(32, 24)
    seeds = scenes.pass_seeds(3, 2)
    sid = renderer.upload(s)
    renderer.set_camera(s.cam)
    aid = renderer.alloc_accum(32, 24)
    renderer.render_passes(sid, aid, seeds, reset_first=1, cfg=s.cfg)
    acc = renderer.read_accum(aid)
    tm = renderer.tonemap(aid)
    ref = O.tonemap(acc)
    assert np.array_equal(tm.view(np.int32), ref.view(np.int32))
    # into a caller's buffer (reused frame after frame): the same bits; a wrong shape is refused
    out = np.full((24, 32, 4), np.nan, np.float32)
    assert renderer.tonemap(aid, out=out) is out
    assert np.array_equal(out.view(np.int32), ref.view(np.int32))
    with pytest.raises(ValueError):
        renderer.tonemap(aid, out=np.zeros((32, 24, 4), np.float32))


def test_block_tiling_covers_frame(renderer):
    """Rendering the four tiles of a 2x2 block grid equals one full-frame pass
    (udpt.cl:166-167, src/RendererCore.cpp:276-307)."""
    s = scenes.c0(37, 29)
    sid = renderer.upload(s)
    renderer.set_camera(s.cam)
    a_full = renderer.alloc_accum(37, 29)
    a_tile = renderer.alloc_accum(37, 29)
    renderer.render(sid, a_full, 4242, reset=1, cfg=s.cfg)
    for b in range(4):
        renderer.render(sid, a_tile, 4242, reset=1, cfg=dict(s.cfg, block=b, block_x=2, block_y=2))
    assert np.array_equal(renderer.read_accum(a_full), renderer.read_accum(a_tile))


@pytest.mark.parametrize("bounces,lights", [(8, 1), (20, 1), (8, 4)])
def test_render_parity_bdpt(renderer, bounces, lights):
    """Naive BDPT (kernels/legacy/bdpt.cl) on the GPU against the oracle."""
    s = scenes.c0_bdpt(40, 32, bounces=bounces, lights=lights)
    seeds = scenes.pass_seeds(8, 2)
    sid = renderer.upload(s)
    renderer.set_camera(s.cam)
    aid = renderer.alloc_accum(40, 32)
    renderer.reset_stats()
    renderer.render_passes(sid, aid, seeds, reset_first=1, cfg=s.cfg)
    gpu = renderer.read_accum(aid)
    st = renderer.stats()
    renderer.free_accum(aid)
    renderer.release(sid)
    ref = np.zeros((32, 40, 4), np.float32)
    for k, sd in enumerate(seeds):
        O.render_bdpt(s, ref, sd, 1 if k == 0 else 0, bounces)
    assert st["stack_overflow"] == 0
    assert _rel_bad(gpu, ref) == 0
    assert np.array_equal(gpu[..., 3], ref[..., 3])
    assert st["samples"] == 40 * 32 * 2


@pytest.mark.parametrize("lights", [1, 4])
def test_bdpt_shade_sort_gives_the_same_pass(renderer, lights):
    """BDPT with every round's shade queue sorted by path state and material class
    (threshold of one path): every pixel against the oracle, the ray count unchanged."""
    s = scenes.c0_bdpt(1024, 512, bounces=8, lights=lights)   # large enough a frame to be sorted
    seeds = scenes.pass_seeds(13, 1)
    sid = renderer.upload(s)
    renderer.set_camera(s.cam)
    renderer.set_shade_sort(1)
    renderer.reset_stats()
    renderer.set_profiling(True)
    aid = renderer.alloc_accum(1024, 512)
    renderer.render_passes(sid, aid, seeds, reset_first=1, cfg=s.cfg)
    gpu = renderer.read_accum(aid)
    st = renderer.stats()
    kt = renderer.kernel_times()
    renderer.set_profiling(False)
    renderer.set_shade_sort(65536)
    renderer.free_accum(aid)
    renderer.release(sid)
    assert kt["sort_launches"] > 0
    ref = np.zeros((512, 1024, 4), np.float32)
    rays = 0
    for k, sd in enumerate(seeds):
        rays += O.render_bdpt(s, ref, sd, 1 if k == 0 else 0, 8, threads=0)["rays"]
    assert _rel_bad(gpu, ref) == 0
    assert np.array_equal(gpu[..., 3], ref[..., 3])
    assert st["rays"] == rays


def test_render_obj_scene(renderer, tmp_path):
    """A scene read from OBJ/MTL files (yh_scene_load_obj) renders like any other: every
    pixel of two passes equals the oracle's (udpt.cl as shipped; the glass material of the
    file is specular and transmissive)."""
    import importlib.util
    import os
    spec = importlib.util.spec_from_file_location("obj_files", os.path.join(os.path.dirname(__file__), "golden",
                                                                            "obj_files.py"))
    objf = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(objf)
    light = scenes.reference_light()
    light["pos"] = (-0.2, 0.9, -0.2, 1.0)
    cam = scenes.camera(eye=(0.0, 0.0, 3.0))
    s = scenes.from_obj(objf.write(str(tmp_path)), 40, 32, lights=light, cam=cam)
    seeds = scenes.pass_seeds(23, 2)
    sid = renderer.upload(s)
    renderer.set_camera(s.cam)
    aid = renderer.alloc_accum(40, 32)
    renderer.render_passes(sid, aid, seeds, reset_first=1, cfg=s.cfg)
    gpu = renderer.read_accum(aid)
    renderer.free_accum(aid)
    renderer.release(sid)
    ref = np.zeros((32, 40, 4), np.float32)
    for k, sd in enumerate(seeds):
        O.render(s, ref, sd, 1 if k == 0 else 0, s.cfg)
    assert np.array_equal(gpu.view(np.int32), ref.view(np.int32))
    assert np.isfinite(gpu).all() and gpu[..., :3].max() > 0.0


def test_save_image_round_trip(renderer, tmp_path):
    """Renderer.save_image (RendererCore::saveImage without GL): the PNG holds the 8-bit
    conversion of the tonemapped frame, rows flipped; the HDR the accumulator's radiance."""
    import zlib
    s = scenes.c0(40, 24)
    sid = renderer.upload(s)
    renderer.set_camera(s.cam)
    aid = renderer.alloc_accum(40, 24)
    renderer.render_passes(sid, aid, scenes.pass_seeds(5, 2), reset_first=1, cfg=s.cfg)
    renderer.save_image(aid, tmp_path / "f.png")
    renderer.save_image(aid, tmp_path / "f.hdr")
    ldr = renderer.tonemap(aid)
    acc = renderer.read_accum(aid)
    renderer.free_accum(aid)
    renderer.release(sid)
    data = open(tmp_path / "f.png", "rb").read()
    idat = data[data.index(b"IDAT") + 4:data.index(b"IEND") - 8]
    raw = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(24, 40 * 3 + 1)[:, 1:].reshape(24, 40, 3)
    want = np.floor(np.clip(np.nan_to_num(ldr[::-1, :, :3]), 0, 1) * np.float32(255) + np.float32(0.5))
    assert np.array_equal(raw, want.astype(np.uint8))
    px = open(tmp_path / "f.hdr", "rb").read().split(b"\n\n", 1)[1].split(b"\n", 1)[1]
    rgbe = np.frombuffer(px, np.uint8).reshape(24, 40, 4).astype(np.float64)
    dec = np.where(rgbe[..., 3:] > 0, rgbe[..., :3] * np.ldexp(1.0, (rgbe[..., 3:] - 136).astype(int)), 0.0)
    ref = acc[::-1, :, :3].astype(np.float64)
    assert (np.abs(dec - ref) <= ref.max(axis=-1, keepdims=True) * 2.0 ** -7 + 1e-30).all()


def test_c4_stress_scene_bdpt_parity(renderer):
    """The stress scene itself (10,004,490 triangles, 8.5M reference nodes, four lights,
    BDPT with 8 vertices per subpath, then the bidirectional tracer with MIS, paths of at
    most 8 segments) on a 32 x 18 crop of the frame, two passes: every pixel and the ray
    counts against the oracle. The oracle's breadth-first queue is
    raised so that no hit is dropped (the core's walk has no such limit)."""
    s = scenes.c4(32, 18)
    assert s.n_tri == 10_004_490
    seeds = scenes.pass_seeds(44, 2)
    sid = renderer.upload(s)
    renderer.set_camera(s.cam)
    aid = renderer.alloc_accum(32, 18)
    out = []
    # the naive BDPT of the configuration, then the bidirectional tracer with MIS
    for cfg in (s.cfg, dict(s.cfg, integrator=2)):
        renderer.reset_stats()
        renderer.render_passes(sid, aid, seeds, reset_first=1, cfg=cfg)
        out.append((renderer.read_accum(aid), renderer.stats()))
    renderer.free_accum(aid)
    renderer.release(sid)
    for (gpu, st), mis in zip(out, (False, True)):
        ref = np.zeros((18, 32, 4), np.float32)
        rays = 0
        for k, sd in enumerate(seeds):
            if mis:
                c = O.render_bdpt_mis(s, ref, sd, 1 if k == 0 else 0, 8, s.cfg, heap_size=1 << 22)
            else:
                c = O.render_bdpt(s, ref, sd, 1 if k == 0 else 0, 8, heap_size=1 << 22)
            assert c["heap_overflow"] == 0
            rays += c["rays"]
        assert st["stack_overflow"] == 0
        assert _rel_bad(gpu, ref) == 0
        assert np.array_equal(gpu[..., 3], ref[..., 3])
        assert st["rays"] == rays


@pytest.mark.parametrize("tree", [0, 2])
def test_render_identical_across_tree_modes(renderer, tree):
    """Every interior hierarchy gives the reference's hits, so whole renders are the same
    bits as with the default one."""
    s = scenes.c1(40, 32, level=5)
    seeds = scenes.pass_seeds(21, 2)
    out = []
    for mode in (1, tree):
        renderer.set_tree_mode(mode)
        sid = renderer.upload(s)
        renderer.set_tree_mode(1)
        renderer.set_camera(s.cam)
        aid = renderer.alloc_accum(40, 32)
        renderer.reset_stats()
        renderer.render_passes(sid, aid, seeds, reset_first=1, cfg=s.cfg)
        out.append((renderer.read_accum(aid), renderer.stats()))
        renderer.free_accum(aid)
        renderer.release(sid)
    assert out[1][1]["stack_overflow"] == 0
    assert np.array_equal(out[0][0].view(np.int32), out[1][0].view(np.int32))
    assert out[0][1]["rays"] == out[1][1]["rays"]


@pytest.mark.parametrize("tree", [1, 2])
def test_render_identical_with_and_without_mixed_trace(renderer, tree):
    """One traversal launch over a round's closest-hit and any-hit rays (the default)
    gives the same bits and the same ray counts as one launch per kind, and both equal
    the oracle."""
    s = scenes.c1(40, 32, level=5)
    seeds = scenes.pass_seeds(31, 2)
    renderer.set_tree_mode(tree)
    sid = renderer.upload(s)
    renderer.set_tree_mode(1)
    renderer.set_camera(s.cam)
    out = []
    for mixed in (1, 0):
        renderer.set_mixed_trace(mixed)
        aid = renderer.alloc_accum(40, 32)
        renderer.reset_stats()
        renderer.render_passes(sid, aid, seeds, reset_first=1, cfg=s.cfg)
        out.append((renderer.read_accum(aid), renderer.stats()))
        renderer.free_accum(aid)
    renderer.set_mixed_trace(1)
    renderer.release(sid)
    ref = np.zeros((32, 40, 4), np.float32)
    for k, sd in enumerate(seeds):
        O.render(s, ref, sd, 1 if k == 0 else 0, s.cfg)
    for img, st in out:
        assert st["stack_overflow"] == 0
        assert np.array_equal(img.view(np.int32), ref.view(np.int32))
    # (boxes and triangles tested may differ: the speculative walk of a lane depends on
    # which rays share its warp)
    for key in ("rays", "ext_rays", "any_rays", "traversed"):
        assert out[0][1][key] == out[1][1][key], key


@pytest.mark.parametrize("key", [(3, 2), (1, 0), (0, 3)])
def test_ray_sort_gives_the_same_pass(renderer, key):
    """Sorting each round's rays by origin and direction cell before the trace (forced on
    every round here) changes no bit and no ray count; both equal the oracle."""
    s = scenes.c1(48, 40, level=5)
    seeds = scenes.pass_seeds(17, 2)
    sid = renderer.upload(s)
    renderer.set_camera(s.cam)
    out = []
    for ob, db, min_rays in ((0, 0, 65536), (key[0], key[1], 1)):
        renderer.set_ray_sort(ob, db, min_rays)
        renderer.reset_stats()
        renderer.set_profiling(True)
        aid = renderer.alloc_accum(48, 40)
        renderer.render_passes(sid, aid, seeds, reset_first=1, cfg=s.cfg)
        out.append((renderer.read_accum(aid), renderer.stats(), renderer.kernel_times()))
        renderer.set_profiling(False)
        renderer.free_accum(aid)
    renderer.set_ray_sort(3, 2, 65536)
    renderer.release(sid)
    assert out[0][2]["raysort_launches"] == 0 and out[1][2]["raysort_launches"] > 0
    ref = np.zeros((40, 48, 4), np.float32)
    for k, sd in enumerate(seeds):
        O.render(s, ref, sd, 1 if k == 0 else 0, s.cfg)
    for img, st, _ in out:
        assert st["stack_overflow"] == 0
        assert np.array_equal(img.view(np.int32), ref.view(np.int32))
    for k in ("rays", "ext_rays", "any_rays", "traversed"):
        assert out[0][1][k] == out[1][1][k], k


def test_shade_sort_gives_the_same_pass(renderer):
    """Sorting every round's shade queue by path phase and material class (forced with a
    threshold of one path) changes no bit and no ray count of yc_render_pass."""
    s = scenes.c1(1024, 512, level=5)   # large enough a frame to be sorted
    seeds = scenes.pass_seeds(19, 1)
    sid = renderer.upload(s)
    renderer.set_camera(s.cam)
    out = []
    for min_paths in (0, 1):
        renderer.set_shade_sort(min_paths)
        renderer.reset_stats()
        renderer.set_profiling(True)
        aid = renderer.alloc_accum(1024, 512)
        renderer.render_passes(sid, aid, seeds, reset_first=1, cfg=s.cfg)
        out.append((renderer.read_accum(aid), renderer.stats(), renderer.kernel_times()))
        renderer.set_profiling(False)
        renderer.free_accum(aid)
    renderer.set_shade_sort(65536)
    renderer.release(sid)
    assert out[0][2]["sort_launches"] == 0 and out[1][2]["sort_launches"] > 0
    ref = np.zeros((512, 1024, 4), np.float32)
    for k, sd in enumerate(seeds):
        O.render(s, ref, sd, 1 if k == 0 else 0, s.cfg)
    for img, st, _ in out:
        assert np.array_equal(img.view(np.int32), ref.view(np.int32))
    for k in ("rays", "ext_rays", "any_rays", "traversed", "samples"):
        assert out[0][1][k] == out[1][1][k], k


@pytest.mark.parametrize("tree", [1, 2])
def test_tail_kernel_gives_the_same_pass(renderer, tree):
    """Finishing the last paths a thread each (YC_OPT_TAIL) changes no bit of the pass and
    no ray count: off, from 64 paths, and from one resident launch (the default)."""
    s = scenes.c1(48, 40, level=5)
    seeds = scenes.pass_seeds(8, 3)
    renderer.set_tree_mode(tree)
    sid = renderer.upload(s)
    renderer.set_tree_mode(1)
    renderer.set_camera(s.cam)
    out = []
    for tail in (0, 64, -1):
        renderer.set_tail_paths(tail)
        aid = renderer.alloc_accum(48, 40)
        renderer.reset_stats()
        renderer.render_passes(sid, aid, seeds, reset_first=1, cfg=s.cfg)
        out.append((renderer.read_accum(aid), renderer.stats()))
        renderer.free_accum(aid)
    renderer.set_tail_paths(-1)
    renderer.release(sid)
    for img, st in out[1:]:
        assert np.array_equal(img.view(np.int32), out[0][0].view(np.int32))
        for k in ("rays", "extension", "shadow", "mis", "samples", "ext_rays", "any_rays", "stack_overflow"):
            assert st[k] == out[0][1][k], k


def test_checkpoint_resume_is_exact(renderer, tmp_path):
    """A snapshot of the accumulator after three passes, loaded into a fresh accumulator of
    a new context, continues to the same bits as the uninterrupted render."""
    s = scenes.c1(40, 32, level=4)
    seeds = scenes.pass_seeds(61, 5)
    sid = renderer.upload(s)
    renderer.set_camera(s.cam)
    aid = renderer.alloc_accum(40, 32)
    renderer.render_passes(sid, aid, seeds[:3], reset_first=1, cfg=s.cfg)
    renderer.save_checkpoint(aid, tmp_path / "ck.npz", next_pass=3)
    renderer.render_passes(sid, aid, seeds[3:], reset_first=0, cfg=s.cfg)
    whole = renderer.read_accum(aid)
    renderer.free_accum(aid)
    renderer.release(sid)
    with Renderer(0) as r2:
        sid2 = r2.upload(s)
        r2.set_camera(s.cam)
        aid2, meta = r2.load_checkpoint(tmp_path / "ck.npz")
        assert int(meta["next_pass"]) == 3
        r2.render_passes(sid2, aid2, seeds[int(meta["next_pass"]):], reset_first=0, cfg=s.cfg)
        resumed = r2.read_accum(aid2)
    assert np.array_equal(resumed.view(np.int32), whole.view(np.int32))
    assert np.all(whole[..., 3] == 5)


@pytest.mark.parametrize("integrator", [0, 1, 2])
def test_nan_material_is_flagged_pink(renderer, integrator):
    """A material with a NaN emission: the samples through it are NaN and the pixels
    take the reference's PINK sentinel (udpt.cl:193-194), on the GPU as in the oracle."""
    s = scenes.c0(40, 32)
    s.mats = s.mats.copy()
    s.mats[3]["ke"][:3] = np.nan   # the Phong box
    if integrator == 1:
        s.cfg = dict(s.cfg, integrator=1, mis=0, bdpt_bounces=8)
    elif integrator == 2:
        s.cfg = dict(s.cfg, integrator=2, bdpt_bounces=8)
    seeds = scenes.pass_seeds(17, 1)
    sid = renderer.upload(s)
    renderer.set_camera(s.cam)
    aid = renderer.alloc_accum(40, 32)
    renderer.render_passes(sid, aid, seeds, reset_first=1, cfg=s.cfg)
    gpu = renderer.read_accum(aid)
    renderer.free_accum(aid)
    renderer.release(sid)
    ref = np.zeros((32, 40, 4), np.float32)
    if integrator == 0:
        O.render(s, ref, seeds[0], 1, s.cfg)
    elif integrator == 1:
        O.render_bdpt(s, ref, seeds[0], 1, 8)
    else:
        O.render_bdpt_mis(s, ref, seeds[0], 1, 8, s.cfg)
    pink = np.all(np.abs(gpu[..., :3] - np.array([0.988, 0.0588, 0.7529], np.float32)) < 1e-6, axis=-1)
    assert pink.sum() > 0 and not np.isnan(gpu).any()
    assert np.array_equal(gpu.view(np.int32), ref.view(np.int32))


@pytest.mark.parametrize("case", ["brute_force", "no_triangles", "one_pixel", "one_row"])
def test_render_edge_cases(renderer, case):
    """Inputs at the edges of the contract, every pixel against the oracle: no BVH
    (bvh_size = 0: the reference tests every triangle, udpt.cl:277-283), a scene without
    triangles (only the quad light), a 1 x 1 frame and a 33 x 1 frame."""
    w, h = {"one_pixel": (1, 1), "one_row": (33, 1)}.get(case, (24, 20))
    s = scenes.c0(w, h)
    if case == "brute_force":
        s.nodes = s.nodes[:0]
    elif case == "no_triangles":
        s.tris, s.nodes = s.tris[:0], s.nodes[:0]
    seeds = scenes.pass_seeds(29, 2)
    sid = renderer.upload(s)
    renderer.set_camera(s.cam)
    aid = renderer.alloc_accum(w, h)
    renderer.reset_stats()
    renderer.render_passes(sid, aid, seeds, reset_first=1, cfg=s.cfg)
    gpu = renderer.read_accum(aid)
    st = renderer.stats()
    renderer.free_accum(aid)
    renderer.release(sid)
    ref = np.zeros((h, w, 4), np.float32)
    rays = 0
    for k, sd in enumerate(seeds):
        rays += O.render(s, ref, sd, 1 if k == 0 else 0, s.cfg)["rays"]
    assert np.array_equal(gpu.view(np.int32), ref.view(np.int32))
    assert st["rays"] == rays and st["samples"] == w * h * 2


@pytest.mark.parametrize("tree", [1, 2])
def test_render_identical_with_a_split_walk_stack(renderer, tree):
    """YC_OPT_STACK_SMEM: with only 2 or 12 (the default, 0) walk-stack entries in shared
    memory (the rest in the context's spill area) a pass gives the oracle's bits and the
    same ray counts as with the whole stack in shared memory (64)."""
    s = scenes.c1(40, 32, level=5)
    seeds = scenes.pass_seeds(37, 2)
    renderer.set_tree_mode(tree)
    sid = renderer.upload(s)
    renderer.set_tree_mode(1)
    renderer.set_camera(s.cam)
    out = []
    for smem in (64, 2, 12, 0):
        renderer.set_stack_smem(smem)
        aid = renderer.alloc_accum(40, 32)
        renderer.reset_stats()
        renderer.render_passes(sid, aid, seeds, reset_first=1, cfg=s.cfg)
        out.append((renderer.read_accum(aid), renderer.stats()))
        renderer.free_accum(aid)
    renderer.set_stack_smem(0)
    renderer.release(sid)
    ref = np.zeros((32, 40, 4), np.float32)
    for k, sd in enumerate(seeds):
        O.render(s, ref, sd, 1 if k == 0 else 0, s.cfg)
    for img, st in out:
        assert st["stack_overflow"] == 0
        assert st["rays"] == out[0][1]["rays"]
        assert np.array_equal(img.view(np.int32), ref.view(np.int32))
