"""Seeded procedural scenes and the render configurations built from them.

These replace Yune's OBJ/MTL input (src/Scene.cpp:133-383) for headless runs. The
geometry comes from the host producers in libyune_gb300.so (yh_scene_*), the BVH from
yh_bvh_build (the node array of src/BVH.cpp:56-173) and the camera from yh_camera_look
(src/Camera.cpp:66-117).

Configurations (sizes and spp of the benchmark workloads):
  c0  Cornell box: 5 walls (10 tris), two seeded-yaw boxes (24 tris), quad light
      (emission 15) under the ceiling; walls Oren-Nayar sigma^2 = 0.09 (sigma 0.3), one
      box modified Phong exponent 50; 512x512, 64 spp; NEE + MIS, roulette after
      bounce 3; leaf <= 10, 20 bins.
  c1  c0 plus a level-6 icosphere (81,920 tris, radius 0.35) of dielectric IOR 1.5;
      leaf <= 4; 1024x1024, 256 spp, at most 16 bounces, roulette after bounce 3.
  c4  stress: 40 x 40 grid of displaced level-4/5 icospheres (10,004,480 tris) with mixed
      materials on the Cornell floor, four quad lights; naive BDPT, 8 vertices per
      subpath; 3840x2160, 128 spp; leaf <= 4.
  c0_mis, c0_bdpt_mis, c4_mis
      the scenes of c0, c0_bdpt and c4 with the bidirectional tracer with multiple
      importance sampling (YC_BDPT_MIS): paths of at most 20, 8 and 8 segments.
"""
import contextlib
import ctypes as C
import hashlib
import json
import os
from dataclasses import dataclass, field

import numpy as np

from . import _native as N
from .layouts import BVH_NODE, CAM, MATERIAL, QUAD_LIGHT, TRIANGLE, ptr


# Where the scene arrays come from: the library whose yh_scene_* and yh_camera_look entry
# points Builder and camera() call, and the BVH builder of build_bvh. By default both are
# libyune_gb300.so's. A process that must not load the product library -- the CPU
# baseline, which runs the reference's own code -- swaps in another library with the same
# producer entry points and the reference's BVH::createBVH (producers() below); the
# arrays are the same bytes either way.
_producers = {"lib": None, "bvh": None}


def _host():
    return _producers["lib"] if _producers["lib"] is not None else N.lib()


@contextlib.contextmanager
def producers(lib, bvh):
    """Within the block, scenes are generated by `lib` (a ctypes library exporting the
    yh_scene_* and yh_camera_look functions of include/yune_host.h with their argtypes
    set) and BVHs built by `bvh(tris, bins, leaf) -> (nodes, depth)`."""
    old = dict(_producers)
    _producers.update(lib=lib, bvh=bvh)
    try:
        yield
    finally:
        _producers.update(old)


@dataclass
class SceneData:
    tris: np.ndarray
    mats: np.ndarray
    lights: np.ndarray
    nodes: np.ndarray
    depth: int
    cam: np.ndarray
    width: int
    height: int
    spp: int
    cfg: dict = field(default_factory=dict)
    name: str = ""

    @property
    def n_tri(self):
        return len(self.tris)


def default_cfg(**kw):
    cfg = dict(integrator=0, mis=1, rr_threshold=3, max_depth=100000, brdf_model=1, mis_lobe_fix=1,
               bdpt_bounces=20, block=0, block_x=1, block_y=1)
    cfg.update(kw)
    return cfg


def material(kd=(0.3, 0.3, 0.3), ks=(0, 0, 0), ke=(0, 0, 0), n=1.0, px=1.0, py=1.0, alpha=100.0,
             specular=0, transmissive=0):
    m = np.zeros(1, MATERIAL)
    m["ke"] = (*ke, 1.0)
    m["kd"] = (*kd, 1.0)
    m["ks"] = (*ks, 1.0)
    m["n"] = n
    m["k"] = 1.0
    m["px"] = px
    m["py"] = py
    m["alpha_x"] = alpha
    m["alpha_y"] = alpha
    m["is_specular"] = specular
    m["is_transmissive"] = transmissive
    return m


class Builder:
    """Thin owner of a yh_scene handle."""

    def __init__(self):
        self.L = L = _host()
        h = C.c_void_p()
        N.check_host(L.yh_scene_new(C.byref(h)), "yh_scene_new")
        self.h = h

    def __del__(self):
        if getattr(self, "h", None):
            self.L.yh_scene_free(self.h)
            self.h = None

    def cornell(self, seed=0, sigma2=0.09, phong_exp=50.0, emission=15.0, boxes=True):
        N.check_host(self.L.yh_scene_add_cornell(self.h, seed, sigma2, phong_exp, emission, int(boxes)), "cornell")
        return self

    def add_material(self, m):
        mid = C.c_int()
        N.check_host(self.L.yh_scene_add_material(self.h, ptr(m), C.byref(mid)), "material")
        return mid.value

    def icosphere(self, center, radius, level, mat_id, disp=0.0, seed=0):
        c = np.asarray(center, np.float32)
        N.check_host(self.L.yh_scene_add_icosphere(self.h, ptr(c), radius, level, disp, seed, mat_id), "icosphere")
        return self

    def load_obj(self, path):
        """Appends an OBJ file and its material file (yh_scene_load_obj, the rules of
        Scene::loadModel); returns the number of triangles read."""
        n = C.c_int()
        N.check_host(self.L.yh_scene_load_obj(self.h, os.fsencode(path), C.byref(n)), "yh_scene_load_obj " + str(path))
        return n.value

    def add_light(self, l):
        N.check_host(self.L.yh_scene_add_light(self.h, ptr(l)), "light")
        return self

    def arrays(self):
        nt, nm, nl = C.c_int(), C.c_int(), C.c_int()
        L = self.L
        N.check_host(L.yh_scene_counts(self.h, C.byref(nt), C.byref(nm), C.byref(nl)), "counts")
        tris = np.zeros(nt.value, TRIANGLE)
        mats = np.zeros(nm.value, MATERIAL)
        lights = np.zeros(nl.value, QUAD_LIGHT)
        N.check_host(L.yh_scene_copy(self.h, ptr(tris), ptr(mats), ptr(lights)), "copy")
        return tris, mats, lights


def build_bvh(tris, bins=20, leaf=10):
    """Node array of BVH::createBVH for these triangles, and the tree depth."""
    if _producers["bvh"] is not None:
        return _producers["bvh"](tris, bins, leaf)
    L = N.lib()
    h = C.c_void_p()
    N.check_host(L.yh_bvh_build(ptr(tris), len(tris), bins, leaf, C.byref(h)), "yh_bvh_build")
    try:
        n = L.yh_bvh_node_count(h)
        nodes = np.zeros(n, BVH_NODE)
        N.check_host(L.yh_bvh_copy_nodes(h, ptr(nodes), n), "copy nodes")
        depth = L.yh_bvh_depth(h)
    finally:
        L.yh_bvh_free(h)
    return nodes, depth


def layout(s, tree_mode=1):
    """The device layout scene `s` takes once uploaded in tree mode `tree_mode`, computed by
    the upload's repack on the host without a device (yc_scene_layout): a dict of
    device_bytes, node_bytes, stream_bytes, shade_bytes, digest, depth, wide."""
    out = N.SceneLayout()
    tris, nodes = np.ascontiguousarray(s.tris), np.ascontiguousarray(s.nodes)
    N.check(N.lib().yc_scene_layout(ptr(tris), len(tris), len(s.mats), ptr(nodes), len(nodes), tree_mode,
                                    C.byref(out)), "yc_scene_layout")
    return {k: int(getattr(out, k)) for k in ("device_bytes", "node_bytes", "stream_bytes", "shade_bytes", "digest",
                                              "depth", "wide")}


def device_bytes(s, tree_mode=1):
    """Bytes scene `s` will hold on the device once uploaded in tree mode `tree_mode`
    (yc_scene_layout: the upload's repack, run on the host without a device)."""
    return layout(s, tree_mode)["device_bytes"]


def walk_counts(s, rays9, any_hit=False, tree_mode=1):
    """The traversal's algorithmic work on explicit rays, replayed on the host
    (yc_walk_counts): (child boxes tested, triangles tested, per-ray triangle, per-ray t)."""
    tris, nodes = np.ascontiguousarray(s.tris), np.ascontiguousarray(s.nodes)
    rays9 = np.ascontiguousarray(rays9, np.float32)
    n = len(rays9)
    tri = np.zeros(n, np.int32)
    t = np.zeros(n, np.float32)
    b, tt = C.c_uint64(), C.c_uint64()
    N.check(N.lib().yc_walk_counts(ptr(tris), len(tris), ptr(nodes), len(nodes), tree_mode, ptr(rays9), n,
                                   int(any_hit), C.byref(b), C.byref(tt), ptr(tri), ptr(t)), "yc_walk_counts")
    return int(b.value), int(tt.value), tri, t


def set_host_threads(n):
    """Limits the host threads of the BVH builder, the scene cache and the upload's repack
    (yh_set_host_threads; 0 = every core). Their outputs do not depend on it. Returns the
    count now in effect."""
    N.check_host(N.lib().yh_set_host_threads(int(n)), "yh_set_host_threads")
    return N.lib().yh_get_host_threads()


def refit_bvh(tris, nodes):
    """A copy of `nodes` refitted to the (moved) triangles `tris` (yh_bvh_refit): the tree
    of the original build with every box recomputed bottom-up from the new positions."""
    out = np.ascontiguousarray(nodes).copy()
    tris = np.ascontiguousarray(tris)
    N.check_host(N.lib().yh_bvh_refit(ptr(tris), len(tris), ptr(out), len(out)), "yh_bvh_refit")
    return out


def camera(eye=(0.0, 0.0, 1.4), side=(1.0, 0.0, 0.0), up=(0.0, 1.0, 0.0), look=(0.0, 0.0, -1.0), fov=60.0):
    cam = np.zeros(1, CAM)
    a = [np.asarray(v, np.float32) for v in (eye, side, up, look)]
    N.check_host(_host().yh_camera_look(ptr(a[0]), ptr(a[1]), ptr(a[2]), ptr(a[3]), fov, ptr(cam)), "camera")
    return cam


def dielectric(ior=1.5, r0=0.04):
    return material(kd=(0, 0, 0), ks=(r0, r0, r0), n=ior, specular=1, transmissive=1, alpha=0.0)


def reference_light():
    """The one quad light compiled into Yune's kernels (kernels/legacy/udpt.cl:97-106),
    placed for the reference's Cornell-box OBJ: corner (-0.1979, 0.92, -3.1972), facing -y,
    edges 0.4 along x and z, emission 16."""
    l = np.zeros(1, QUAD_LIGHT)
    l["pos"] = (-0.1979, 0.92, -3.1972, 1.0)
    l["normal"] = (0.0, -1.0, 0.0, 0.0)
    l["ke"] = (16.0, 16.0, 16.0, 0.0)
    l["edge_l"] = (0.4, 0.0, 0.0, 0.0)
    l["edge_w"] = (0.0, 0.0, 0.4, 0.0)
    return l


def from_obj(path, width=512, height=512, spp=64, lights=None, cam=None, bins=20, leaf=10, cfg=None):
    """A scene loaded from an OBJ/MTL pair as Yune loads it (Scene::loadModel; BVH with the
    reference's 20 bins and leaves of up to 10 triangles by default). Lights default to
    the reference kernel's quad light, the camera to Yune's default camera (eye at the
    origin looking down -z, 60 degree vertical field of view)."""
    b = Builder()
    b.load_obj(path)
    tris, mats, _ = b.arrays()
    nodes, depth = build_bvh(tris, bins, leaf)
    return SceneData(tris, mats, reference_light() if lights is None else lights, nodes, depth,
                     camera(eye=(0.0, 0.0, 0.0)) if cam is None else cam, width, height, spp,
                     cfg or default_cfg(mis=0, rr_threshold=6, brdf_model=0, mis_lobe_fix=0), "obj")


def c0(width=512, height=512, spp=64, seed=0):
    b = Builder().cornell(seed=seed)
    tris, mats, lights = b.arrays()
    nodes, depth = build_bvh(tris, 20, 10)
    return SceneData(tris, mats, lights, nodes, depth, camera(), width, height, spp,
                     default_cfg(max_depth=100000), "c0")


def c1(width=1024, height=1024, spp=256, seed=0, level=6):
    b = Builder().cornell(seed=seed)
    glass = b.add_material(dielectric(1.5))
    b.icosphere((0.0, 0.0, 0.0), 0.35, level, glass)
    tris, mats, lights = b.arrays()
    nodes, depth = build_bvh(tris, 20, 4)
    return SceneData(tris, mats, lights, nodes, depth, camera(), width, height, spp, default_cfg(max_depth=16), "c1")


def four_lights(lights, emission=(4.0, 7.0, 10.0, 13.0)):
    """Four quad lights under the ceiling, spread across the box (the stress
    configuration's multi-light set, picked per sample by the multiple-light CDF of
    sampleLights, kernels/legacy/udpt.cl:632-698)."""
    out = np.zeros(4, QUAD_LIGHT)
    for i in range(4):
        out[i] = lights[0]
        out[i]["pos"][0] = -0.4 + 0.22 * i
        out[i]["pos"][2] = -0.3 + 0.1 * i
        out[i]["ke"][:3] = emission[i]
    return out


def c0_bdpt(width=512, height=512, spp=64, seed=0, bounces=8, lights=4):
    """Cornell box with `lights` quad lights, naive BDPT with `bounces` vertices per
    subpath (the stress configuration's integrator on the small scene)."""
    b = Builder().cornell(seed=seed)
    tris, mats, ls = b.arrays()
    if lights == 4:
        ls = four_lights(ls)
    nodes, depth = build_bvh(tris, 20, 10)
    return SceneData(tris, mats, ls, nodes, depth, camera(), width, height, spp,
                     default_cfg(integrator=1, mis=0, bdpt_bounces=bounces), "c0_bdpt")


def c4(width=3840, height=2160, spp=128, seed=0, grid=40, n_level5=118, bounces=8):
    """The stress configuration: a flattened grid x grid array of displaced icospheres on
    the floor of the Cornell box (walls only), four quad lights under the ceiling, naive
    BDPT with `bounces` vertices per subpath.

    Sphere levels: `n_level5` seeded spheres of level 5 (20,480 triangles) and the rest of
    level 4 (5,120), so the 40 x 40 grid holds 10,004,480 sphere triangles, the stated
    10M (a grid of 1,600 level-6 spheres would hold 131M). Each sphere: radius 0.4 of the
    grid pitch, vertices moved radially by U(-5%, 5%) of the radius, one material drawn
    uniformly from {Oren-Nayar, modified Phong with exponent in [10, 200], dielectric
    with IOR in [1.3, 1.7]}. All draws come from numpy's PCG64 stream of `seed`."""
    from .workloads import random_material
    rng = np.random.default_rng(seed)
    b = Builder().cornell(seed=seed, boxes=False)
    pitch = 0.9 / grid
    r = 0.4 * pitch
    big = set(rng.choice(grid * grid, size=min(n_level5, grid * grid), replace=False).tolist())
    for i in range(grid):
        for j in range(grid):
            k = i * grid + j
            mid = b.add_material(random_material(rng))
            c = (-0.45 + (j + 0.5) * pitch, -0.5 + r * 1.06, -0.45 + (i + 0.5) * pitch)
            b.icosphere(c, r, 5 if k in big else 4, mid, disp=0.05, seed=seed * 1000003 + k)
    tris, mats, ls = b.arrays()
    ls = four_lights(ls)
    nodes, depth = build_bvh(tris, 20, 4)
    look = np.array([0.0, -0.45, -1.0])
    look /= np.linalg.norm(look)
    up = np.array([0.0, -look[2], look[1]])
    cam = camera(eye=(0.0, 0.2, 1.3), side=(1.0, 0.0, 0.0), up=tuple(up), look=tuple(look), fov=50.0)
    return SceneData(tris, mats, ls, nodes, depth, cam, width, height, spp,
                     default_cfg(integrator=1, mis=0, bdpt_bounces=bounces), "c4")


def _with_mis(s, name, kmax):
    s.cfg = dict(s.cfg, integrator=2, bdpt_bounces=kmax)
    s.name = name
    return s


def c0_mis(width=512, height=512, spp=64, seed=0, kmax=20):
    """c0's scene and options rendered by the bidirectional tracer with MIS, paths of at
    most kmax segments (the unidirectional c0 is unbounded; 20 segments leave out a
    fraction of about 1e-5 of the radiance)."""
    return _with_mis(c0(width, height, spp, seed), "c0_mis", kmax)


def c0_bdpt_mis(width=512, height=512, spp=64, seed=0, bounces=8, lights=4):
    """c0_bdpt's scene (four lights) with the bidirectional tracer with MIS, paths of at
    most `bounces` segments."""
    return _with_mis(c0_bdpt(width, height, spp, seed, bounces, lights), "c0_bdpt_mis", bounces)


def c4_mis(width=3840, height=2160, spp=128, seed=0, bounces=8):
    """The stress scene with the bidirectional tracer with MIS, paths of at most `bounces`
    segments."""
    return _with_mis(c4(width, height, spp, seed, bounces=bounces), "c4_mis", bounces)


CONFIGS = {"c0": c0, "c1": c1, "c0_bdpt": c0_bdpt, "c4": c4, "c0_mis": c0_mis, "c0_bdpt_mis": c0_bdpt_mis,
           "c4_mis": c4_mis}


# ---- binary scene cache (yh_cache_*) ----
# Part of every cache key: raise it when a generator's output changes, so that files
# written by the old generator read as stale instead of standing in for the new scene.
CACHE_GENERATION = 1


def cache_key(name, **params):
    """64-bit key of configuration `name` built with `params` (and CACHE_GENERATION)."""
    text = json.dumps([CACHE_GENERATION, name, sorted(params.items())], sort_keys=True)
    return int.from_bytes(hashlib.sha256(text.encode()).digest()[:8], "little")


def save_cache(s, path, key):
    """Writes scene `s` to the binary scene cache file `path` under `key` (yh_cache_save):
    its arrays, BVH and camera, and its frame size, spp, options and name as the file's
    caller bytes."""
    meta = json.dumps(dict(width=s.width, height=s.height, spp=s.spp, cfg=s.cfg, name=s.name)).encode()
    arrs = [np.ascontiguousarray(a) for a in (s.tris, s.mats, s.lights, s.nodes, s.cam)]
    tris, mats, lights, nodes, cam = arrs
    if cam.nbytes != CAM.itemsize:
        raise ValueError("the scene's camera must be one Cam record")
    N.check_host(N.lib().yh_cache_save(os.fsencode(path), key, ptr(tris), len(tris), ptr(mats), len(mats),
                                       ptr(lights), len(lights), ptr(nodes), len(nodes), int(s.depth), ptr(cam),
                                       meta, len(meta)), "yh_cache_save " + str(path))


def load_cache(path, key):
    """The SceneData written by save_cache to `path` (yh_cache_load). Raises YuneError with
    code YH_E_STALE when the file was made for another key, YH_E_FORMAT when it is not an
    intact cache file, YH_E_IO when it cannot be read."""
    L = N.lib()
    info = N.CacheInfo()
    N.check_host(L.yh_cache_query(os.fsencode(path), C.byref(info)), "yh_cache_query " + str(path))
    if info.key != key:
        raise N.YuneError(N.YH_E_STALE, "yh_cache_load %s: %s" % (path, N.HOST_ERRORS[N.YH_E_STALE]))
    tris = np.empty(info.n_tri, TRIANGLE)
    mats = np.empty(info.n_mat, MATERIAL)
    lights = np.empty(info.n_light, QUAD_LIGHT)
    nodes = np.empty(info.n_node, BVH_NODE)
    cam = np.empty(1, CAM)
    meta = C.create_string_buffer(max(1, info.meta_bytes))
    N.check_host(L.yh_cache_load(os.fsencode(path), key, ptr(tris), len(tris), ptr(mats), len(mats), ptr(lights),
                                 len(lights), ptr(nodes), len(nodes), ptr(cam) if info.has_cam else None,
                                 meta, info.meta_bytes), "yh_cache_load " + str(path))
    m = json.loads(meta.raw[:info.meta_bytes].decode()) if info.meta_bytes else {}
    if not info.has_cam:
        cam = camera()
    return SceneData(tris, mats, lights, nodes, info.depth, cam, int(m.get("width", 512)), int(m.get("height", 512)),
                     int(m.get("spp", 64)), dict(m.get("cfg", default_cfg())), str(m.get("name", "")))


def cached(name, path, **params):
    """CONFIGS[name](**params) through the cache file `path`: read back when the file holds
    that configuration with those parameters, otherwise built and written there (a missing,
    stale or damaged file is replaced)."""
    key = cache_key(name, **params)
    try:
        return load_cache(path, key)
    except N.YuneError as e:
        if e.code not in (N.YH_E_IO, N.YH_E_FORMAT, N.YH_E_STALE):
            raise
    s = CONFIGS[name](**params)
    save_cache(s, path, key)
    return s


def pass_seeds(seed, n):
    """Per-pass `rand` values: the first n outputs of std::mt19937(seed), which is what
    uniform_int_distribution<unsigned>(0, UINT_MAX) over mt19937 returns
    (src/RendererCore.cpp:61-63, 268)."""
    return mt19937(seed, n)


def mt19937(seed, n):
    """First n outputs of the 32-bit Mersenne Twister (Matsumoto and Nishimura 1998)."""
    mt = [0] * 624
    mt[0] = seed & 0xFFFFFFFF
    for i in range(1, 624):
        mt[i] = (1812433253 * (mt[i - 1] ^ (mt[i - 1] >> 30)) + i) & 0xFFFFFFFF
    idx = 624
    out = []
    for _ in range(n):
        if idx >= 624:
            for i in range(624):
                y = (mt[i] & 0x80000000) | (mt[(i + 1) % 624] & 0x7FFFFFFF)
                mt[i] = mt[(i + 397) % 624] ^ (y >> 1) ^ (0x9908B0DF if y & 1 else 0)
            idx = 0
        y = mt[idx]
        idx += 1
        y ^= y >> 11
        y ^= (y << 7) & 0x9D2C5680
        y ^= (y << 15) & 0xEFC60000
        y ^= y >> 18
        out.append(y & 0xFFFFFFFF)
    return np.array(out, dtype=np.uint32)


def box_rays(n, seed=0):
    """n incoherent rays as 9 float32 each (origin xyz 1, direction xyz 0, length inf):
    origins uniform inside the Cornell box, directions uniform on the sphere (numpy's
    PCG64 stream of `seed`)."""
    rng = np.random.default_rng(seed)
    o = rng.uniform(-0.49, 0.49, size=(n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3))
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    r = np.zeros((n, 9), np.float32)
    r[:, 0:3] = o
    r[:, 3] = 1.0
    r[:, 4:7] = d
    r[:, 8] = np.inf
    return r
