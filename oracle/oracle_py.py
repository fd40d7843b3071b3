"""ctypes front end of the CPU oracle (liboracle.so) and of the compiled reference
(_ref/libyune_ref.so).

TEST INFRASTRUCTURE: used by tests, the smoke check and the benchmark's CPU-baseline
leg only.
"""
import ctypes as C
import os

import numpy as np

from . import build_oracle

vp = C.c_void_p
i32 = C.c_int
u32 = C.c_uint32


class OrCfg(C.Structure):
    _fields_ = [("mis", i32), ("rr_threshold", i32), ("max_depth", i32), ("brdf_model", i32),
                ("mis_lobe_fix", i32), ("heap_size", i32), ("gi_check", i32)]


class OrCounters(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in ("rays", "primary", "extension", "shadow", "mis", "heap_overflow")]


_orc = None
_ref = None
_ref_tried = False


def _p(a):
    return None if a is None else a.ctypes.data


def orc():
    global _orc
    if _orc is None:
        path = build_oracle.build_oracle()
        L = C.CDLL(path)
        L.or_trace.argtypes = [vp, i32, vp, i32, vp, i32, vp, i32, i32, i32, vp, vp, vp, vp]
        L.or_render.argtypes = [vp, i32, vp, i32, vp, i32, vp, i32, vp, i32, i32, vp, u32, i32, C.POINTER(OrCfg), i32,
                                i32, i32, C.POINTER(OrCounters)]
        L.or_render_f64.argtypes = L.or_render.argtypes
        L.or_render_bdpt.argtypes = [vp, i32, vp, i32, vp, i32, vp, i32, vp, i32, i32, vp, u32, i32,
                                     C.POINTER(OrCfg), i32, i32, i32, i32, C.POINTER(OrCounters)]
        L.or_render_bdpt_f64.argtypes = L.or_render_bdpt.argtypes
        L.or_render_bdpt_mis.argtypes = L.or_render_bdpt.argtypes
        L.or_render_bdpt_mis_f64.argtypes = L.or_render_bdpt.argtypes
        L.or_tonemap.argtypes = [vp, i32, i32, vp]
        L.or_ym_eval.argtypes = [i32, vp, vp, vp, i32]
        L.or_wang_hash.argtypes = [u32]
        L.or_wang_hash.restype = u32
        L.or_xor_shift.argtypes = [u32]
        L.or_xor_shift.restype = u32
        L.or_render_pixels_f64.argtypes = [vp, i32, vp, i32, vp, i32, vp, i32, vp, i32, i32, vp, vp, i32, vp, i32,
                                           C.POINTER(OrCfg), i32, i32, vp, i32]
        L.or_brdf.argtypes = [vp, i32, vp, i32, i32, vp, vp, vp, vp, i32, C.c_float, i32, vp]
        L.or_record_rays.argtypes = [vp, i32, vp, i32, vp, i32, vp, i32, vp, i32, i32, u32, C.POINTER(OrCfg), i32,
                                     i32, vp, C.c_int64, C.POINTER(C.c_int64)]
        _orc = L
    return _orc


def ref():
    """The compiled reference, or None when no reference text is available."""
    global _ref, _ref_tried
    if not _ref_tried:
        _ref_tried = True
        _ref = _load_ref(False)
    return _ref


_ref_libm = None
_ref_libm_tried = False


def ref_libm():
    """The compiled reference with the host C library's cosf, sinf and powf as its built-ins,
    or None when no reference text is available."""
    global _ref_libm, _ref_libm_tried
    if not _ref_libm_tried:
        _ref_libm_tried = True
        _ref_libm = _load_ref(True)
    return _ref_libm


def _load_ref(libm):
    try:
        path = build_oracle.build_ref(libm=libm)
    except RuntimeError:
        path = None
    if not (path and os.path.exists(path)):
        return None
    L = C.CDLL(path)
    L.ref_render.argtypes = [i32, vp, i32, vp, i32, vp, i32, vp, i32, vp, i32, i32, vp, u32, i32, i32, i32, i32, i32,
                             i32, i32]
    L.ref_trace.argtypes = [vp, i32, vp, i32, vp, i32, vp, i32, i32, vp, vp, vp]
    L.ref_tonemap.argtypes = [vp, i32, i32, vp]
    L.ref_oren_nayar.argtypes = [vp, vp, vp, vp, vp, vp]
    if hasattr(L, "ref_bvh_build"):
        L.ref_bvh_build.argtypes = [vp, i32, i32, i32, vp, i32, C.POINTER(i32)]
    if hasattr(L, "ref_load_obj"):
        L.ref_load_obj.argtypes = [C.c_char_p, C.c_char_p, vp, i32, C.POINTER(i32), vp, i32, C.POINTER(i32), vp,
                                   i32, C.POINTER(i32)]
    return L


_scene_lib = None


def scene_lib():
    """The oracle library's copy of the procedural scene producers (yh_scene_* and
    yh_camera_look, the same sources as the product's), with argtypes set: the CPU
    baseline generates its inputs with it, so it never loads the product library."""
    global _scene_lib
    if _scene_lib is None:
        L = orc()
        f = C.c_float
        sig = {"yh_scene_new": (i32, [C.POINTER(vp)]), "yh_scene_free": (None, [vp]),
               "yh_scene_add_material": (i32, [vp, vp, C.POINTER(i32)]),
               "yh_scene_add_cornell": (i32, [vp, C.c_uint64, f, f, f, i32]),
               "yh_scene_add_icosphere": (i32, [vp, vp, f, i32, f, C.c_uint64, i32]),
               "yh_scene_add_light": (i32, [vp, vp]),
               "yh_scene_counts": (i32, [vp, C.POINTER(i32), C.POINTER(i32), C.POINTER(i32)]),
               "yh_scene_copy": (i32, [vp, vp, vp, vp]),
               "yh_scene_load_obj": (i32, [vp, C.c_char_p, C.POINTER(i32)]),
               "yh_camera_look": (i32, [vp, vp, vp, vp, f, vp])}
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _scene_lib = L
    return _scene_lib


def node_depth(nodes):
    """Longest root-to-leaf path (edges) of a reference node array (children of an
    interior node at child_idx and child_idx + 1)."""
    n = len(nodes)
    if n == 0:
        return 0
    child = nodes["child_idx"].astype(np.int64)
    depth = np.zeros(n, np.int64)
    for i in range(n):   # breadth-first order: a parent precedes its children
        c = child[i]
        if c > 0 and c + 1 < n:
            depth[c] = depth[c + 1] = depth[i] + 1
    return int(depth.max())


def ref_bvh_with_depth(tris, bins=20, leaf=10):
    """BVH::createBVH of the compiled reference (src/BVH.cpp), and the tree depth."""
    nodes = ref_bvh(tris, bins, leaf)
    return nodes, node_depth(nodes)


def cfg_of(cfg, heap_size=1500):
    c = OrCfg()
    c.mis = int(cfg.get("mis", 0))
    c.rr_threshold = int(cfg.get("rr_threshold", 6))
    c.max_depth = int(cfg.get("max_depth", 100000))
    c.brdf_model = int(cfg.get("brdf_model", 0))
    c.mis_lobe_fix = int(cfg.get("mis_lobe_fix", 0))
    c.heap_size = heap_size
    c.gi_check = int(cfg.get("gi_check", 1))
    return c


def render(scene, accum, rand_seed, reset, cfg, threads=0, rows=None, f64=False, heap_size=1500):
    """One oracle pass into accum (H x W x 4, float32 or float64 for f64)."""
    L = orc()
    H, W = accum.shape[:2]
    cnt = OrCounters()
    c = cfg_of(cfg, heap_size)
    r0, r1 = rows if rows else (0, 0)
    fn = L.or_render_f64 if f64 else L.or_render
    rc = fn(_p(scene.tris), len(scene.tris), _p(scene.mats), len(scene.mats), _p(scene.nodes), len(scene.nodes),
            _p(scene.lights), len(scene.lights), _p(scene.cam), W, H, _p(accum), int(rand_seed) & 0xFFFFFFFF, reset,
            C.byref(c), threads, r0, r1, C.byref(cnt))
    if rc != 0:
        raise RuntimeError("or_render failed: %d" % rc)
    return {k: getattr(cnt, k) for k, _ in OrCounters._fields_}


def record_rays(scene, rand_seed, cfg, rows, cap=1 << 22):
    """The rays one oracle pass over `rows` (y0, y1) walks a BVH with, as the CUDA core
    walks them (a shadow ray a light closes first and a MIS ray that misses the sampled
    light settle without a walk): (n, 8) float32, origin xyz, direction xyz, length,
    kind (0 camera, 1 extension: closest hit; 2 shadow, 3 MIS: any hit)."""
    L = orc()
    out = np.zeros((cap, 8), np.float32)
    n = C.c_int64()
    c = cfg_of(cfg)
    rc = L.or_record_rays(_p(scene.tris), len(scene.tris), _p(scene.mats), len(scene.mats), _p(scene.nodes),
                          len(scene.nodes), _p(scene.lights), len(scene.lights), _p(scene.cam), scene.width,
                          scene.height, int(rand_seed) & 0xFFFFFFFF, C.byref(c), rows[0], rows[1], _p(out), cap,
                          C.byref(n))
    if rc != 0:
        raise RuntimeError("or_record_rays failed")
    return out[:min(n.value, cap)].copy()


def rays9_of(rec):
    """Recorded rays in the 9-float ray format (origin xyzw, dir xyzw, length)."""
    r = np.zeros((len(rec), 9), np.float32)
    r[:, 0:3] = rec[:, 0:3]
    r[:, 3] = 1.0
    r[:, 4:7] = rec[:, 3:6]
    r[:, 8] = rec[:, 6]
    return r


def render_bdpt(scene, accum, rand_seed, reset, bounces, threads=0, rows=None, f64=False, heap_size=1500):
    """One oracle BDPT pass (bdpt.cl) into accum."""
    L = orc()
    H, W = accum.shape[:2]
    cnt = OrCounters()
    c = cfg_of({}, heap_size)
    r0, r1 = rows if rows else (0, 0)
    fn = L.or_render_bdpt_f64 if f64 else L.or_render_bdpt
    rc = fn(_p(scene.tris), len(scene.tris), _p(scene.mats), len(scene.mats), _p(scene.nodes), len(scene.nodes),
            _p(scene.lights), len(scene.lights), _p(scene.cam), W, H, _p(accum), int(rand_seed) & 0xFFFFFFFF, reset,
            C.byref(c), bounces, threads, r0, r1, C.byref(cnt))
    if rc != 0:
        raise RuntimeError("or_render_bdpt failed: %d" % rc)
    return {k: getattr(cnt, k) for k, _ in OrCounters._fields_}


def render_bdpt_mis(scene, accum, rand_seed, reset, kmax, cfg, threads=0, rows=None, f64=False, heap_size=1500):
    """One pass of the bidirectional tracer with multiple importance sampling
    (bdpt_mis_oracle.hpp) into accum; cfg supplies rr_threshold and brdf_model."""
    L = orc()
    H, W = accum.shape[:2]
    cnt = OrCounters()
    c = cfg_of(cfg, heap_size)
    r0, r1 = rows if rows else (0, 0)
    fn = L.or_render_bdpt_mis_f64 if f64 else L.or_render_bdpt_mis
    rc = fn(_p(scene.tris), len(scene.tris), _p(scene.mats), len(scene.mats), _p(scene.nodes), len(scene.nodes),
            _p(scene.lights), len(scene.lights), _p(scene.cam), W, H, _p(accum), int(rand_seed) & 0xFFFFFFFF, reset,
            C.byref(c), kmax, threads, r0, r1, C.byref(cnt))
    if rc != 0:
        raise RuntimeError("or_render_bdpt_mis failed: %d" % rc)
    return {k: getattr(cnt, k) for k, _ in OrCounters._fields_}


def reference_pixels_f64(scene, xs, ys, seeds, cfg, bdpt_bounces=0, threads=0, bdpt_mis=False):
    """FP64 running mean over len(seeds) passes at the given pixels (n x 4 doubles);
    bdpt_mis selects the bidirectional tracer with multiple importance sampling, with
    paths of at most bdpt_bounces segments."""
    L = orc()
    xs = np.ascontiguousarray(xs, np.int32)
    ys = np.ascontiguousarray(ys, np.int32)
    sd = np.ascontiguousarray(seeds, np.uint32)
    out = np.zeros((len(xs), 4), np.float64)
    c = cfg_of(cfg)
    rc = L.or_render_pixels_f64(_p(scene.tris), len(scene.tris), _p(scene.mats), len(scene.mats), _p(scene.nodes),
                                len(scene.nodes), _p(scene.lights), len(scene.lights), _p(scene.cam), scene.width,
                                scene.height, _p(xs), _p(ys), len(xs), _p(sd), len(sd), C.byref(c), bdpt_bounces,
                                threads, _p(out), int(bool(bdpt_mis)))
    if rc != 0:
        raise RuntimeError("or_render_pixels_f64 failed")
    return out


def trace(scene, rays9, any_hit=False, heap_size=1500):
    L = orc()
    rays9 = np.ascontiguousarray(rays9, np.float32)
    n = rays9.shape[0]
    tri = np.zeros(n, np.int32)
    light = np.zeros(n, np.int32)
    t = np.zeros(n, np.float32)
    ov = np.zeros(n, np.int32)
    rc = L.or_trace(_p(scene.tris), len(scene.tris), _p(scene.nodes), len(scene.nodes), _p(scene.lights),
                    len(scene.lights), _p(rays9), n, int(any_hit), heap_size, _p(tri), _p(light), _p(t), _p(ov))
    if rc != 0:
        raise RuntimeError("or_trace failed")
    return tri, light, t, ov


def tonemap(accum):
    L = orc()
    H, W = accum.shape[:2]
    out = np.zeros((H, W, 4), np.float32)
    a = np.ascontiguousarray(accum, np.float32)
    L.or_tonemap(_p(a), W, H, _p(out))
    return out


# ---- the compiled reference ----
VARIANT = {"udpt_a": 0, "udpt_mis": 1, "udpt_mis4": 2, "udpt_mis_on": 3, "bdpt20": 10, "bdpt8": 11, "bdpt8_l4": 12}


def ref_render(scene, accum, rand_seed, reset, variant, rr_threshold, max_depth, gi_check=1, threads=0, rows=None,
               libm=False):
    L = ref_libm() if libm else ref()
    H, W = accum.shape[:2]
    r0, r1 = rows if rows else (0, 0)
    rc = L.ref_render(VARIANT[variant], _p(scene.tris), len(scene.tris), _p(scene.mats), len(scene.mats),
                      _p(scene.nodes), len(scene.nodes), _p(scene.lights), len(scene.lights), _p(scene.cam), W, H,
                      _p(accum), int(rand_seed) & 0xFFFFFFFF, reset, gi_check, rr_threshold, max_depth, threads, r0,
                      r1)
    if rc != 0:
        raise RuntimeError("ref_render failed: %d" % rc)


def ref_trace(scene, rays9, any_hit=False):
    L = ref()
    rays9 = np.ascontiguousarray(rays9, np.float32)
    n = rays9.shape[0]
    tri = np.zeros(n, np.int32)
    light = np.zeros(n, np.int32)
    t = np.zeros(n, np.float32)
    rc = L.ref_trace(_p(scene.tris), len(scene.tris), _p(scene.nodes), len(scene.nodes), _p(scene.lights),
                     len(scene.lights), _p(rays9), n, int(any_hit), _p(tri), _p(light), _p(t))
    if rc != 0:
        raise RuntimeError("ref_trace failed: %d" % rc)
    return tri, light, t


def ref_load_obj(path, cap_tris=1 << 20, cap_nodes=1 << 21, cap_mats=1024):
    """Scene::loadModel of the compiled reference on an OBJ file: (triangles, materials,
    BVH nodes) as the reference leaves them in Scene::vert_data, mat_data and
    bvh.gpu_node_list (20 bins, leaf <= 10)."""
    from yune_gb300.layouts import BVH_NODE, MATERIAL, TRIANGLE
    L = ref()
    if L is None or not hasattr(L, "ref_load_obj"):
        raise RuntimeError("compiled reference loader not available")
    tris = np.zeros(cap_tris, TRIANGLE)
    mats = np.zeros(cap_mats, MATERIAL)
    nodes = np.zeros(cap_nodes, BVH_NODE)
    nt, nm, nn = i32(), i32(), i32()
    rc = L.ref_load_obj(os.fsencode(path), os.fsencode(os.path.basename(path)), _p(tris), cap_tris, C.byref(nt),
                        _p(mats), cap_mats, C.byref(nm), _p(nodes), cap_nodes, C.byref(nn))
    if rc != 0:
        raise RuntimeError("ref_load_obj failed: %d" % rc)
    return tris[:nt.value].copy(), mats[:nm.value].copy(), nodes[:nn.value].copy()


def ref_tonemap(accum):
    L = ref()
    H, W = accum.shape[:2]
    out = np.zeros((H, W, 4), np.float32)
    a = np.ascontiguousarray(accum, np.float32)
    L.ref_tonemap(_p(a), W, H, _p(out))
    return out


def ref_bvh(tris, bins=20, leaf=10):
    from yune_gb300.layouts import BVH_NODE
    L = ref()
    cap = max(64, 8 * len(tris))
    out = np.zeros(cap, BVH_NODE)
    n = C.c_int()
    rc = L.ref_bvh_build(_p(tris), len(tris), bins, leaf, _p(out), cap, C.byref(n))
    if rc != 0:
        raise RuntimeError("ref_bvh_build failed: %d" % rc)
    return out[: n.value].copy()


def seeded_rays(scene, n, seed=0, inside=True):
    """n rays (origin xyzw, dir xyzw, length) with origins inside the scene box and
    directions uniform on the sphere, as 9 float32 per ray; w = 1 for origins and 0 for
    directions, as the reference's rays carry."""
    rng = np.random.default_rng(seed)
    lo = np.array([-0.49, -0.49, -0.49])
    hi = np.array([0.49, 0.49, 0.49])
    o = rng.uniform(lo, hi, size=(n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    d = d.astype(np.float32)
    r = np.zeros((n, 9), np.float32)
    r[:, 0:3] = o
    r[:, 3] = 1.0
    r[:, 4:7] = d
    r[:, 7] = 0.0
    r[:, 8] = np.inf
    return r
