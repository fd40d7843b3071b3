"""The CPU oracle and the host producers against Yune's own code.

Two sources of truth: the golden fixtures in tests/golden (made by make_golden.py from
the reference kernels and BVH builder compiled as C++), which travel everywhere, and
the compiled reference itself where the reference tree is present (more cases).
Everything here is bit-exact.
"""
import os

import numpy as np
import pytest

from oracle import oracle_py as O
from yune_gb300 import scenes

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load(name):
    return np.load(os.path.join(GOLD, name), allow_pickle=False)


def _gold_scenes():
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLD, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    return mg, mg.golden_scenes()


MG, SCENES = _gold_scenes()


@pytest.mark.parametrize("name", sorted(SCENES))
def test_scene_generator_matches_fixture(name):
    g = _load("bvh_%s.npz" % name)
    assert MG.scene_hash(SCENES[name]) == str(g["scene_sha256"]), "procedural scene drifted from the fixture"


@pytest.mark.parametrize("name", sorted(SCENES))
def test_bvh_builder_matches_reference(name):
    g = _load("bvh_%s.npz" % name)
    s = SCENES[name]
    nodes, _ = scenes.build_bvh(s.tris, int(g["bins"]), int(g["leaf"]))
    f = MG.node_fields(nodes)
    for k in ("child_idx", "vert_len", "vert_list", "p_min", "p_max"):
        assert np.array_equal(np.asarray(f[k]).view(np.int32), np.asarray(g[k]).view(np.int32)), k


@pytest.fixture(scope="module")
def large_scene():
    return MG.large_scene()


@pytest.mark.parametrize("threads", [0, 1, 3, 16])
@pytest.mark.parametrize("leaf", [4, 10])
def test_bvh_builder_large_matches_reference(large_scene, leaf, threads):
    """A scene large enough that the host builder splits single nodes over threads: the
    node array equals BVH::createBVH's (digest of the compiled reference's) whatever the
    number of host threads (0: all cores)."""
    from yune_gb300 import _native as N
    g = _load("bvh_large.npz")
    assert MG.scene_hash(large_scene) == str(g["scene_sha256"]), "procedural scene drifted from the fixture"
    L = N.lib()
    assert L.yh_set_host_threads(threads) == 0
    try:
        assert L.yh_get_host_threads() == threads if threads else L.yh_get_host_threads() >= 1
        nodes, _ = scenes.build_bvh(large_scene.tris, int(g["bins"]), leaf)
    finally:
        L.yh_set_host_threads(0)
    assert len(nodes) == int(g["nodes_leaf%d" % leaf])
    assert MG.node_digest(nodes) == str(g["digest_leaf%d" % leaf])


@pytest.mark.parametrize("name", sorted(SCENES))
def test_oracle_trace_matches_reference(name):
    g = _load("trace_%s.npz" % name)
    s = SCENES[name]
    rays = O.seeded_rays(s, int(g["n_rays"]), seed=int(g["ray_seed"]))
    tri, light, t, ov = O.trace(s, rays)
    assert ov.sum() == 0
    assert np.array_equal(tri, g["tri"]) and np.array_equal(light, g["light"])
    assert np.array_equal(t.view(np.int32), g["t"].view(np.int32))
    seg = rays.copy()
    seg[:, 8] = np.where(np.isfinite(t), t * np.float32(1.001), np.float32(0.6))
    a_tri, a_light, _, _ = O.trace(s, seg, any_hit=True)
    assert np.array_equal((a_tri >= 0) | (a_light >= 0), g["occluded"])


def test_oracle_render_and_tonemap_match_reference():
    g = _load("render_c0.npz")
    s = SCENES["c0"]
    seeds = g["seeds"]
    for variant, cfg in (("udpt_a", dict(mis=0, rr_threshold=6, max_depth=100000)),
                         ("udpt_mis", dict(mis=1, rr_threshold=3, max_depth=100000))):
        acc = np.zeros((24, 32, 4), np.float32)
        for k, sd in enumerate(seeds):
            O.render(s, acc, sd, 1 if k == 0 else 0, cfg, threads=2)
        assert np.array_equal(acc.view(np.int32), g[variant].view(np.int32)), variant
    tm = O.tonemap(g["udpt_mis"])
    assert np.array_equal(tm.view(np.int32), g["tonemap_mis"].view(np.int32))


def test_oracle_oren_nayar_matches_reference():
    g = _load("oren_nayar.npz")
    m = g["material"]
    n = len(g["value"])
    from yune_gb300.layouts import TRIANGLE
    tri = np.zeros(1, TRIANGLE)
    tri["matID"] = 0
    L = O.orc()
    out = np.zeros((n, 4), np.float32)
    for i in range(n):
        o = np.zeros(4, np.float32)
        hp = np.ascontiguousarray(g["hit_point"][i])
        nr = np.ascontiguousarray(g["normal"][i])
        wi = np.ascontiguousarray(g["w_i"][i])
        wo = np.ascontiguousarray(g["w_o"][i])
        L.or_brdf(tri.ctypes.data, 1, m.ctypes.data, 1, 0, hp.ctypes.data, nr.ctypes.data, wi.ctypes.data,
                  wo.ctypes.data, 0, 1.0, 1, o.ctypes.data)
        out[i] = o
    assert np.array_equal(out.view(np.int32), g["value"].view(np.int32))


@pytest.mark.parametrize("name", sorted(MG.VARIANT_B))
def test_oracle_variant_b_matches_reference(name):
    """The restatement with brdf_model 1 (Oren-Nayar) and no lobe fix equals the
    compiled composite udpt.cl -DMIS + udpt-primitives.cl's Oren-Nayar rule."""
    g = _load("render_variant_b.npz")
    s = SCENES[name]
    assert MG.scene_hash(s) == str(g[name + "_sha256"])
    v = MG.VARIANT_B[name]
    cfg = dict(mis=1, rr_threshold=v["rr"], max_depth=v["max_depth"], brdf_model=1, mis_lobe_fix=0)
    acc = np.zeros((24, 32, 4), np.float32)
    for k, sd in enumerate(g[name + "_seeds"]):
        O.render(s, acc, sd, 1 if k == 0 else 0, cfg, threads=2)
    assert np.array_equal(acc.view(np.int32), g[name].view(np.int32))


@pytest.mark.parametrize("lights", [1, 4])
def test_oracle_bdpt_matches_reference(lights):
    g = _load("render_bdpt.npz")
    s = scenes.c0_bdpt(32, 24, bounces=8, lights=lights)
    assert MG.scene_hash(s) == str(g["sha_lights%d" % lights])
    acc = np.zeros((24, 32, 4), np.float32)
    for k, sd in enumerate(g["seeds"]):
        O.render_bdpt(s, acc, sd, 1 if k == 0 else 0, 8, threads=2)
    assert np.array_equal(acc.view(np.int32), g["lights%d" % lights].view(np.int32))


# ---- live comparisons against the compiled reference (where the reference tree is) ----
needs_ref = pytest.mark.skipif(O.ref() is None, reason="compiled reference not available")
# the reference's host code (BVH builder, loader) is compiled only where its sources are
needs_ref_host = pytest.mark.skipif(O.ref() is None or not hasattr(O.ref(), "ref_bvh_build"),
                                    reason="compiled reference host code not available")


@needs_ref_host
@pytest.mark.parametrize("level,leaf", [(4, 4), (5, 4), (4, 10)])
def test_bvh_builder_live(level, leaf):
    s = scenes.c1(16, 16, level=level)
    mine, _ = scenes.build_bvh(s.tris, 20, leaf)
    ref = O.ref_bvh(s.tris, 20, leaf)
    a, b = MG.node_fields(mine), MG.node_fields(ref)
    for k in a:
        assert np.array_equal(np.asarray(a[k]).view(np.int32), np.asarray(b[k]).view(np.int32)), k


@needs_ref_host
def test_bvh_builder_median_and_displaced_live():
    b = scenes.Builder().cornell(seed=3)
    mid = b.add_material(scenes.material(kd=(0.5, 0.5, 0.5)))
    b.icosphere((0.1, -0.1, 0.0), 0.3, 4, mid, disp=0.05, seed=17)
    tris, mats, lights = b.arrays()
    for bins in (0, 2, 7, 20, 64):
        mine, _ = scenes.build_bvh(tris, bins, 6)
        ref = O.ref_bvh(tris, bins, 6)
        x, y = MG.node_fields(mine), MG.node_fields(ref)
        for k in x:
            assert np.array_equal(np.asarray(x[k]).view(np.int32), np.asarray(y[k]).view(np.int32)), (bins, k)


@needs_ref
def test_oracle_trace_live_large():
    s = scenes.c1(16, 16, level=5)
    rays = O.seeded_rays(s, 20000, seed=21)
    a = O.trace(s, rays)
    b = O.ref_trace(s, rays)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[2].view(np.int32), b[2].view(np.int32))


@needs_ref
@pytest.mark.parametrize("variant,cfg", [
    ("udpt_a", dict(mis=0, rr_threshold=6, max_depth=100000)),
    ("udpt_mis", dict(mis=1, rr_threshold=3, max_depth=16)),
    ("udpt_mis", dict(mis=1, rr_threshold=0, max_depth=4)),
    # variant B, the configurations' composite: udpt.cl -DMIS with udpt-primitives.cl's
    # Oren-Nayar diffuse rule (the restatement's brdf_model 1, without the lobe fix)
    ("udpt_mis_on", dict(mis=1, rr_threshold=3, max_depth=16, brdf_model=1, mis_lobe_fix=0)),
    ("udpt_mis_on", dict(mis=1, rr_threshold=0, max_depth=100000, brdf_model=1, mis_lobe_fix=0)),
])
def test_oracle_render_live_glass(variant, cfg):
    s = scenes.c1(24, 20, level=4)
    seeds = scenes.pass_seeds(77, 2)
    a = np.zeros((20, 24, 4), np.float32)
    b = np.zeros((20, 24, 4), np.float32)
    for k, sd in enumerate(seeds):
        O.render(s, a, sd, 1 if k == 0 else 0, cfg, threads=4)
        O.ref_render(s, b, sd, 1 if k == 0 else 0, variant, cfg["rr_threshold"], cfg["max_depth"], threads=4)
    assert np.array_equal(a.view(np.int32), b.view(np.int32))


@needs_ref
def test_oracle_render_live_variant_b_cornell():
    """Variant B on the Cornell box, whose walls are Oren-Nayar (sigma^2 0.09) and one box
    modified Phong: every pixel of the restatement equals the compiled composite."""
    s = scenes.c0(32, 24)
    seeds = scenes.pass_seeds(41, 3)
    cfg = dict(mis=1, rr_threshold=3, max_depth=100000, brdf_model=1, mis_lobe_fix=0)
    a = np.zeros((24, 32, 4), np.float32)
    b = np.zeros((24, 32, 4), np.float32)
    for k, sd in enumerate(seeds):
        O.render(s, a, sd, 1 if k == 0 else 0, cfg, threads=4)
        O.ref_render(s, b, sd, 1 if k == 0 else 0, "udpt_mis_on", 3, 100000, threads=4)
    assert np.array_equal(a.view(np.int32), b.view(np.int32))


@needs_ref
def test_oracle_render_live_brute_force_and_gi_off():
    s = scenes.c0(20, 16)
    s.nodes = s.nodes[:0]
    seeds = scenes.pass_seeds(5, 2)
    for gi in (1, 0):
        a = np.zeros((16, 20, 4), np.float32)
        b = np.zeros((16, 20, 4), np.float32)
        for k, sd in enumerate(seeds):
            O.render(s, a, sd, 1 if k == 0 else 0, dict(mis=0, rr_threshold=6, max_depth=100000, gi_check=gi))
            O.ref_render(s, b, sd, 1 if k == 0 else 0, "udpt_a", 6, 100000, gi_check=gi)
        assert np.array_equal(a.view(np.int32), b.view(np.int32))


@needs_ref
@pytest.mark.parametrize("variant,bounces", [("bdpt20", 20), ("bdpt8", 8)])
def test_oracle_bdpt_live_glass_scene(variant, bounces):
    """BDPT on the icosphere scene (no specular materials in bdpt.cl: the dielectric is
    shaded as its kd/ks say)."""
    s = scenes.c1(24, 20, level=3)
    seeds = scenes.pass_seeds(12, 2)
    a = np.zeros((20, 24, 4), np.float32)
    b = np.zeros((20, 24, 4), np.float32)
    for k, sd in enumerate(seeds):
        O.render_bdpt(s, a, sd, 1 if k == 0 else 0, bounces, threads=4)
        O.ref_render(s, b, sd, 1 if k == 0 else 0, variant, 4, 100000, threads=4)
    assert np.array_equal(a.view(np.int32), b.view(np.int32))
