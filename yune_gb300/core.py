"""RendererCore-style driver over the C-ABI (the calls src/RendererCore.cpp makes).

    r = Renderer()                       # CLManager::setup
    sid = r.upload(scene)                # setupVertexBuffer / setupMatBuffer / setupBVHBuffer
    r.set_camera(scene.cam)              # setupCameraBuffer, Camera::setBuffer
    aid = r.alloc_accum(w, h)            # setupImageBuffers
    r.render(sid, aid, rand, reset=1)    # enqueueKernels: one `pathtracer` pass
    img = r.tonemap(aid)                 # the `tonemap` pass
"""
import ctypes as C
import os
import weakref

import numpy as np

from . import _native as N
from .layouts import ptr


def write_png(path, rgba):
    """8-bit RGB PNG of an (H, W, 4) float frame (yh_write_png), first file row = last frame row."""
    a = np.ascontiguousarray(rgba, np.float32)
    N.check_host(N.lib().yh_write_png(os.fsencode(str(path)), a.shape[1], a.shape[0], ptr(a)), "yh_write_png")


def write_hdr(path, rgba):
    """Radiance RGBE file of an (H, W, 4) float frame (yh_write_hdr)."""
    a = np.ascontiguousarray(rgba, np.float32)
    N.check_host(N.lib().yh_write_hdr(os.fsencode(str(path)), a.shape[1], a.shape[0], ptr(a)), "yh_write_hdr")


def cfg_struct(cfg):
    s = N.PassCfg()
    for k, _ in N.PassCfg._fields_:
        setattr(s, k, int(cfg.get(k, 0)))
    if s.block_x == 0:
        s.block_x = 1
    if s.block_y == 0:
        s.block_y = 1
    return s


class Renderer:
    def __init__(self, device=0):
        self.L = N.lib()
        h = C.c_void_p()
        N.check(self.L.yc_create(device, C.byref(h)), "yc_create")
        self.h = h
        self._accum_shape = {}
        self._children = weakref.WeakSet()   # batches: the context releases them
        self.tree_mode = 1                   # YC_OPT_TREE of later uploads

    def close(self):
        if getattr(self, "h", None):
            for ch in list(self._children):
                ch._detach()
            self.L.yc_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def upload(self, scene):
        sid = C.c_int()
        N.check(self.L.yc_upload_scene(self.h, ptr(scene.tris), len(scene.tris), ptr(scene.mats), len(scene.mats),
                                       ptr(scene.nodes), len(scene.nodes), ptr(scene.lights), len(scene.lights),
                                       C.byref(sid)), "yc_upload_scene")
        return sid.value

    def scene_depth(self, sid):
        d = C.c_int()
        N.check(self.L.yc_scene_depth(self.h, sid, C.byref(d)), "yc_scene_depth")
        return d.value

    def scene_digest(self, sid):
        """Digest of the uploaded scene's repacked arrays as they lie on the device (yc_scene_digest);
        equals `scenes.layout(...).digest` for the same inputs and tree mode."""
        h = C.c_uint64()
        N.check(self.L.yc_scene_digest(self.h, sid, C.byref(h)), "yc_scene_digest")
        return int(h.value)

    def build_bvh(self, tris, bins=20, leaf=10):
        """BVH::createBVH on this renderer's GPU (yc_bvh_build): the node array of
        scenes.build_bvh, and the tree depth."""
        from .layouts import BVH_NODE
        t = np.ascontiguousarray(tris)
        n, d = C.c_int(), C.c_int()
        N.check(self.L.yc_bvh_build(self.h, ptr(t), len(t), int(bins), int(leaf), C.byref(n), C.byref(d)),
                "yc_bvh_build")
        nodes = np.zeros(n.value, BVH_NODE)
        N.check(self.L.yc_bvh_copy_nodes(self.h, ptr(nodes), n.value), "yc_bvh_copy_nodes")
        return nodes, d.value

    def refit(self, sid, tris):
        """Moves the uploaded scene's triangles to `tris` (same triangles, new positions) and
        refits its hierarchy on the device (yc_refit_scene)."""
        t = np.ascontiguousarray(tris)
        N.check(self.L.yc_refit_scene(self.h, sid, ptr(t), len(t)), "yc_refit_scene")

    def scene_bytes(self, sid):
        """Bytes the scene holds on the device."""
        b = C.c_uint64()
        N.check(self.L.yc_scene_bytes(self.h, sid, C.byref(b)), "yc_scene_bytes")
        return int(b.value)

    def release(self, sid):
        N.check(self.L.yc_release_scene(self.h, sid), "yc_release_scene")

    def set_camera(self, cam):
        N.check(self.L.yc_set_camera(self.h, ptr(cam)), "yc_set_camera")

    def alloc_accum(self, w, h):
        aid = C.c_int()
        N.check(self.L.yc_alloc_accum(self.h, w, h, C.byref(aid)), "yc_alloc_accum")
        self._accum_shape[aid.value] = (h, w)
        return aid.value

    def free_accum(self, aid):
        N.check(self.L.yc_free_accum(self.h, aid), "yc_free_accum")
        self._accum_shape.pop(aid, None)

    def render(self, sid, aid, rand_seed, reset=0, gi_check=1, cfg=None):
        c = cfg_struct(cfg or {})
        N.check(self.L.yc_render_pass(self.h, sid, aid, int(rand_seed) & 0xFFFFFFFF, reset, gi_check, C.byref(c)),
                "yc_render_pass")

    def render_passes(self, sid, aid, seeds, reset_first=1, gi_check=1, cfg=None):
        c = cfg_struct(cfg or {})
        s = np.ascontiguousarray(seeds, dtype=np.uint32)
        N.check(self.L.yc_render_passes(self.h, sid, aid, ptr(s), len(s), reset_first, gi_check, C.byref(c)),
                "yc_render_passes")

    def read_accum(self, aid):
        h, w = self._accum_shape[aid]
        out = np.zeros((h, w, 4), np.float32)
        N.check(self.L.yc_read_accum(self.h, aid, ptr(out)), "yc_read_accum")
        return out

    def write_accum(self, aid, img):
        img = np.ascontiguousarray(img, np.float32)
        N.check(self.L.yc_write_accum(self.h, aid, ptr(img)), "yc_write_accum")

    def tonemap(self, aid, out=None):
        """The tonemapped frame (yc_tonemap) as a (h, w, 4) float32 array: a new one, or `out`
        (C-contiguous float32 of that shape, e.g. a page-locked buffer reused frame after
        frame)."""
        h, w = self._accum_shape[aid]
        if out is None:
            out = np.zeros((h, w, 4), np.float32)
        elif out.shape != (h, w, 4) or out.dtype != np.float32 or not out.flags["C_CONTIGUOUS"]:
            raise ValueError("tonemap: out must be a C-contiguous float32 array of shape %s" % ((h, w, 4),))
        N.check(self.L.yc_tonemap(self.h, aid, ptr(out)), "yc_tonemap")
        return out

    def trace(self, sid, rays9, any_hit=False):
        rays9 = np.ascontiguousarray(rays9, np.float32)
        n = rays9.shape[0]
        tri = np.zeros(n, np.int32)
        light = np.zeros(n, np.int32)
        t = np.zeros(n, np.float32)
        N.check(self.L.yc_trace(self.h, sid, ptr(rays9), n, int(any_hit), ptr(tri), ptr(light), ptr(t)), "yc_trace")
        return tri, light, t

    def trace_device(self, sid, rays_ptr, n, any_hit, tri_ptr, t_ptr):
        """yc_trace_device on caller-owned device buffers (9 floats per ray in)."""
        N.check(self.L.yc_trace_device(self.h, sid, C.c_void_p(rays_ptr), n, int(any_hit), C.c_void_p(tri_ptr),
                                       C.c_void_p(t_ptr)), "yc_trace_device")

    def stats(self):
        s = N.Stats()
        N.check(self.L.yc_get_stats(self.h, C.byref(s)), "yc_get_stats")
        return {k: getattr(s, k) for k, _ in N.Stats._fields_}

    def reset_stats(self):
        N.check(self.L.yc_reset_stats(self.h), "yc_reset_stats")

    def last_pass_ms(self):
        ms = C.c_float()
        N.check(self.L.yc_last_pass_ms(self.h, C.byref(ms)), "yc_last_pass_ms")
        return ms.value

    def set_tree_mode(self, mode):
        """0: reference node tree; 1: SAH hierarchy over the reference leaves (default);
        2: the same hierarchy with four-child nodes. Applies to later uploads."""
        N.check(self.L.yc_set_option(self.h, 1, int(mode)), "yc_set_option")
        self.tree_mode = int(mode)

    def event(self, slot):
        """Records event `slot` (0..7) on the context stream after the work queued so far."""
        N.check(self.L.yc_event_record(self.h, int(slot)), "yc_event_record")

    def elapsed_ms(self, a, b):
        """Device milliseconds between recorded events a and b (waits for b)."""
        ms = C.c_float()
        N.check(self.L.yc_event_elapsed_ms(self.h, int(a), int(b), C.byref(ms)), "yc_event_elapsed_ms")
        return ms.value

    def set_max_rounds(self, n):
        """Rounds one pass may take before the call fails with YC_E_TIMEOUT (default 1,000,000)."""
        N.check(self.L.yc_set_option(self.h, 7, int(n)), "yc_set_option")

    def set_stack_limit(self, n):
        """Traversal stack entries a walk may use (0: what the scene needs); a walk that
        reaches the limit fails the call with YC_E_OVERFLOW."""
        N.check(self.L.yc_set_option(self.h, 8, int(n)), "yc_set_option")

    def set_stack_smem(self, n):
        """Walk-stack entries the per-pass traversal keeps in shared memory (YC_OPT_STACK_SMEM;
        the deeper ones go to a spill area in global memory; 0 = 12, the default; 64 or any
        value at or above the scene's stack depth = the whole stack)."""
        N.check(self.L.yc_set_option(self.h, 9, int(n)), "yc_set_option")

    def set_repack(self, on_device):
        """Where later uploads repack a tree-mode-1 scene (YC_OPT_REPACK): 1 on the device
        (default), 0 on the host; the bytes are the same."""
        N.check(self.L.yc_set_option(self.h, 10, int(on_device)), "yc_set_option")

    def set_tail_paths(self, n):
        """Paths left at which a pass finishes in the tail kernel (-1 auto, 0 off)."""
        N.check(self.L.yc_set_option(self.h, 2, int(n)), "yc_set_option")

    def save_image(self, aid, path):
        """RendererCore::saveImage without GL: `.png` writes the tonemapped frame as 8-bit
        RGB, `.hdr` the accumulator's linear radiance as Radiance RGBE."""
        ext = os.path.splitext(str(path))[1].lower()
        if ext == ".png":
            write_png(path, self.tonemap(aid))
        elif ext == ".hdr":
            write_hdr(path, self.read_accum(aid))
        else:
            raise ValueError("image output is .png or .hdr")

    def save_checkpoint(self, aid, path, **meta):
        """Snapshot of an accumulator: its float4 running means with the pass count in w
        (udpt.cl:203-208), so rendering can resume from it in another context or process.
        `meta` (scene name, next pass index, seeds, ...) is stored beside it."""
        np.savez(path, accum=self.read_accum(aid), **{k: np.asarray(v) for k, v in meta.items()})

    def load_checkpoint(self, path):
        """Allocates an accumulator holding a snapshot made by save_checkpoint; returns its
        id and the stored metadata. Passes rendered into it with reset 0 continue the
        running mean exactly where the snapshot left it."""
        with np.load(path) as d:
            acc = d["accum"]
            meta = {k: d[k] for k in d.files if k != "accum"}
        if acc.ndim != 3 or acc.shape[2] != 4:
            raise ValueError("not an accumulator snapshot")
        aid = self.alloc_accum(acc.shape[1], acc.shape[0])
        self.write_accum(aid, acc)
        return aid, meta

    def set_mixed_trace(self, on):
        """1: a round's closest-hit and any-hit rays share one traversal launch (default);
        0: one launch each."""
        N.check(self.L.yc_set_option(self.h, 3, int(on)), "yc_set_option")

    def set_ray_sort(self, origin_bits=3, dir_bits=2, min_rays=None):
        """Sort key of a round's rays before the mixed traversal launch (0, 0: queue
        order); rounds with fewer than min_rays rays stay unsorted."""
        N.check(self.L.yc_set_option(self.h, 4, int(origin_bits) * 10 + int(dir_bits)), "yc_set_option")
        if min_rays is not None:
            N.check(self.L.yc_set_option(self.h, 5, int(min_rays)), "yc_set_option")

    def set_shade_sort(self, min_paths):
        """Per-pass shade queues of at least min_paths paths are sorted by phase and
        material class before shading (0: never)."""
        N.check(self.L.yc_set_option(self.h, 6, int(min_paths)), "yc_set_option")

    def set_profiling(self, on=True):
        N.check(self.L.yc_set_profiling(self.h, int(on)), "yc_set_profiling")

    def kernel_times(self):
        k = N.KernelTimes()
        N.check(self.L.yc_get_kernel_times(self.h, C.byref(k)), "yc_get_kernel_times")
        return {n: getattr(k, n) for n, _ in N.KernelTimes._fields_}

    def flush_l2(self, nbytes=256 << 20):
        N.check(self.L.yc_flush_l2(self.h, nbytes), "yc_flush_l2")

    def measure_l2_gbs(self, nbytes=48 << 20, iters=20):
        g = C.c_double()
        N.check(self.L.yc_measure_l2_gbs(self.h, nbytes, iters, C.byref(g)), "yc_measure_l2_gbs")
        return g.value

    def synchronize(self):
        N.check(self.L.yc_synchronize(self.h), "yc_synchronize")
