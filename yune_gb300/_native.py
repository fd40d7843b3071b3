"""ctypes bindings of libyune_gb300.so (include/yune_cuda.h and include/yune_host.h).

The library is loaded from the package directory only; when it is missing the import
fails with the build command to run, so nothing falls back to another implementation.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libyune_gb300.so")

vp = C.c_void_p
i32 = C.c_int
u32 = C.c_uint32
f32 = C.c_float


class PassCfg(C.Structure):
    """yc_pass_cfg"""
    _fields_ = [("integrator", i32), ("mis", i32), ("rr_threshold", i32), ("max_depth", i32),
                ("brdf_model", i32), ("mis_lobe_fix", i32), ("bdpt_bounces", i32), ("block", i32),
                ("block_x", i32), ("block_y", i32)]


class Stats(C.Structure):
    """yc_stats"""
    _fields_ = [(n, C.c_uint64) for n in ("rays", "primary", "extension", "shadow", "mis", "connection",
                                          "traversed", "samples", "stack_overflow", "ext_rays", "ext_boxes",
                                          "ext_tris", "any_rays", "any_boxes", "any_tris")]


class KernelTimes(C.Structure):
    """yc_kernel_times"""
    _fields_ = [("raygen_ms", C.c_double), ("extend_ms", C.c_double), ("occlusion_ms", C.c_double),
                ("logic_ms", C.c_double), ("raygen_launches", C.c_uint64), ("extend_launches", C.c_uint64),
                ("occlusion_launches", C.c_uint64), ("logic_launches", C.c_uint64), ("rounds", C.c_uint64),
                ("sort_ms", C.c_double), ("sort_launches", C.c_uint64), ("tail_ms", C.c_double),
                ("tail_launches", C.c_uint64), ("trace_ms", C.c_double), ("trace_launches", C.c_uint64),
                ("raysort_ms", C.c_double), ("raysort_launches", C.c_uint64)]


class SceneLayout(C.Structure):
    """yc_scene_layout_info"""
    _fields_ = [("device_bytes", C.c_uint64), ("node_bytes", C.c_uint64), ("stream_bytes", C.c_uint64),
                ("shade_bytes", C.c_uint64), ("digest", C.c_uint64), ("depth", i32), ("wide", i32)]


class CacheInfo(C.Structure):
    """yh_cache_info"""
    _fields_ = [("key", C.c_uint64), ("n_tri", i32), ("n_mat", i32), ("n_light", i32), ("n_node", i32),
                ("depth", i32), ("has_cam", i32), ("meta_bytes", i32)]


class BatchCfg(C.Structure):
    """yc_batch_cfg"""
    _fields_ = [("pool_paths", i32), ("rounds_per_launch", i32), ("logic_blocks_per_sm", i32), ("use_graph", i32),
                ("max_jobs", i32), ("stack_cap", i32), ("sort_threshold", i32), ("groups", i32), ("ray_sort", i32),
                ("trace_block", i32), ("stack_smem", i32), ("trace_share", i32)]


class ServeCfg(C.Structure):
    """yc_serve_cfg"""
    _fields_ = [("budget_bytes", C.c_uint64), ("max_queue", i32), ("keep_results", i32), ("batch", BatchCfg)]


class Cam(C.Structure):
    """yc_cam (80 bytes: rows r1..r4 as float4, view_plane_dist, padding)"""
    _fields_ = [("f", f32 * 20)]


class RequestDesc(C.Structure):
    """yc_request_desc"""
    _fields_ = [("cam", Cam), ("cfg", PassCfg), ("scene_id", i32), ("width", i32), ("height", i32), ("n_pass", i32),
                ("seeds_host", vp)]


class RequestInfo(C.Structure):
    """yc_request_info"""
    _fields_ = [("state", i32), ("accum_id", i32), ("pixels_done", C.c_int64), ("pixels_total", C.c_int64),
                ("submit_s", C.c_double), ("admit_s", C.c_double), ("finish_s", C.c_double)]


class TuneJob(C.Structure):
    """yc_tune_job"""
    _fields_ = [("cam", Cam), ("cfg", PassCfg), ("scene_id", i32), ("width", i32), ("height", i32), ("n_pass", i32),
                ("seeds_host", vp)]


class TuneTrial(C.Structure):
    """yc_tune_trial"""
    _fields_ = [("cfg", BatchCfg), ("ms", f32)]


TUNE_CLOCK = C.CFUNCTYPE(f32, C.POINTER(BatchCfg), vp)   # yc_tune_clock

# request states (YC_REQ_*)
REQ_WAITING, REQ_RUNNING, REQ_CANCELLING, REQ_DONE, REQ_CANCELLED, REQ_REJECTED_BUDGET, REQ_REJECTED_QUEUE = range(7)


# name -> (restype, argtypes)
SIGNATURES = {
    # core
    "yc_create": (i32, [i32, C.POINTER(vp)]),
    "yc_destroy": (i32, [vp]),
    "yc_last_error": (C.c_char_p, []),
    "yc_synchronize": (i32, [vp]),
    "yc_upload_scene": (i32, [vp, vp, i32, vp, i32, vp, i32, vp, i32, C.POINTER(i32)]),
    "yc_set_lights": (i32, [vp, i32, vp, i32]),
    "yc_bvh_build": (i32, [vp, vp, i32, i32, i32, C.POINTER(i32), C.POINTER(i32)]),
    "yc_bvh_copy_nodes": (i32, [vp, vp, i32]),
    "yc_release_scene": (i32, [vp, i32]),
    "yc_refit_scene": (i32, [vp, i32, vp, i32]),
    "yc_scene_bytes": (i32, [vp, i32, C.POINTER(C.c_uint64)]),
    "yc_scene_depth": (i32, [vp, i32, C.POINTER(i32)]),
    "yc_scene_digest": (i32, [vp, i32, C.POINTER(C.c_uint64)]),
    "yc_scene_layout": (i32, [vp, i32, i32, vp, i32, i32, vp]),
    "yc_set_camera": (i32, [vp, vp]),
    "yc_walk_counts": (i32, [vp, i32, vp, i32, i32, vp, i32, i32, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), vp,
                             vp]),
    "yc_alloc_accum": (i32, [vp, i32, i32, C.POINTER(i32)]),
    "yc_free_accum": (i32, [vp, i32]),
    "yc_read_accum": (i32, [vp, i32, vp]),
    "yc_write_accum": (i32, [vp, i32, vp]),
    "yc_accum_device_ptr": (i32, [vp, i32, C.POINTER(vp)]),
    "yc_render_pass": (i32, [vp, i32, i32, u32, i32, i32, C.POINTER(PassCfg)]),
    "yc_render_passes": (i32, [vp, i32, i32, vp, i32, i32, i32, C.POINTER(PassCfg)]),
    "yc_render_pass_noalloc": (i32, [vp, i32, i32, u32, i32, i32, C.POINTER(PassCfg)]),
    "yc_tonemap": (i32, [vp, i32, vp]),
    "yc_trace": (i32, [vp, i32, vp, i32, i32, vp, vp, vp]),
    "yc_trace_device": (i32, [vp, i32, vp, i32, i32, vp, vp]),
    "yc_get_stats": (i32, [vp, C.POINTER(Stats)]),
    "yc_reset_stats": (i32, [vp]),
    "yc_last_pass_ms": (i32, [vp, C.POINTER(f32)]),
    "yc_device_allocations": (i32, [C.POINTER(C.c_uint64)]),
    "yc_event_record": (i32, [vp, i32]),
    "yc_event_elapsed_ms": (i32, [vp, i32, i32, C.POINTER(f32)]),
    "yc_set_profiling": (i32, [vp, i32]),
    "yc_set_option": (i32, [vp, i32, i32]),
    "yc_get_kernel_times": (i32, [vp, C.POINTER(KernelTimes)]),
    "yc_flush_l2": (i32, [vp, C.c_size_t]),
    "yc_measure_l2_gbs": (i32, [vp, C.c_size_t, i32, C.POINTER(C.c_double)]),
    "yc_batch_create": (i32, [vp, C.POINTER(BatchCfg), C.POINTER(vp)]),
    "yc_batch_add_job": (i32, [vp, i32, i32, vp, vp, i32, i32, C.POINTER(PassCfg), C.POINTER(i32)]),
    "yc_batch_run": (i32, [vp, i32, C.POINTER(i32)]),
    "yc_batch_job_progress": (i32, [vp, i32, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "yc_batch_cancel_job": (i32, [vp, i32]),
    "yc_batch_destroy": (i32, [vp]),
    "yc_batch_tune": (i32, [vp, vp, i32, C.POINTER(BatchCfg), i32, C.POINTER(BatchCfg), vp, i32, C.POINTER(i32)]),
    "yc_tune_search": (i32, [C.POINTER(BatchCfg), C.c_int64, i32, vp, vp, C.POINTER(BatchCfg), vp, i32,
                             C.POINTER(i32)]),
    # serving and admission
    "yc_admission_create": (i32, [C.c_uint64, i32, C.POINTER(vp)]),
    "yc_admission_submit": (i32, [vp, C.c_uint64, C.POINTER(C.c_int64), C.POINTER(i32)]),
    "yc_admission_next": (i32, [vp, C.POINTER(C.c_int64)]),
    "yc_admission_cancel": (i32, [vp, C.c_int64, C.POINTER(i32)]),
    "yc_admission_finish": (i32, [vp, C.c_int64, C.POINTER(i32)]),
    "yc_admission_state": (i32, [vp, C.c_int64, C.POINTER(i32)]),
    "yc_admission_usage": (i32, [vp, C.POINTER(C.c_uint64), C.POINTER(i32), C.POINTER(i32)]),
    "yc_admission_destroy": (i32, [vp]),
    "yc_serve_create": (i32, [vp, C.POINTER(ServeCfg), C.POINTER(vp)]),
    "yc_serve_submit": (i32, [vp, C.POINTER(RequestDesc), C.POINTER(C.c_int64), C.POINTER(i32)]),
    "yc_serve_cancel": (i32, [vp, C.c_int64]),
    "yc_serve_step": (i32, [vp, i32, C.POINTER(i32), C.POINTER(i32)]),
    "yc_serve_info": (i32, [vp, C.c_int64, C.POINTER(RequestInfo)]),
    "yc_serve_read": (i32, [vp, C.c_int64, vp]),
    "yc_serve_release": (i32, [vp, C.c_int64]),
    "yc_serve_clock": (C.c_double, [vp]),
    "yc_serve_destroy": (i32, [vp]),
    # host producers
    "yh_bvh_build": (i32, [vp, i32, i32, i32, C.POINTER(vp)]),
    "yh_bvh_node_count": (i32, [vp]),
    "yh_bvh_copy_nodes": (i32, [vp, vp, i32]),
    "yh_bvh_depth": (i32, [vp]),
    "yh_bvh_free": (None, [vp]),
    "yh_bvh_refit": (i32, [vp, i32, vp, i32]),
    "yh_triangle_aabb": (i32, [vp, vp, vp]),
    "yh_camera_look": (i32, [vp, vp, vp, vp, f32, vp]),
    "yh_scene_new": (i32, [C.POINTER(vp)]),
    "yh_scene_free": (None, [vp]),
    "yh_scene_add_material": (i32, [vp, vp, C.POINTER(i32)]),
    "yh_scene_add_cornell": (i32, [vp, C.c_uint64, f32, f32, f32, i32]),
    "yh_scene_add_icosphere": (i32, [vp, vp, f32, i32, f32, C.c_uint64, i32]),
    "yh_scene_add_light": (i32, [vp, vp]),
    "yh_scene_counts": (i32, [vp, C.POINTER(i32), C.POINTER(i32), C.POINTER(i32)]),
    "yh_scene_load_obj": (i32, [vp, C.c_char_p, C.POINTER(i32)]),
    "yh_write_png": (i32, [C.c_char_p, i32, i32, vp]),
    "yh_write_hdr": (i32, [C.c_char_p, i32, i32, vp]),
    "yh_scene_copy": (i32, [vp, vp, vp, vp]),
    "yh_set_host_threads": (i32, [i32]),
    "yh_get_host_threads": (i32, []),
    "yh_cache_save": (i32, [C.c_char_p, C.c_uint64, vp, i32, vp, i32, vp, i32, vp, i32, i32, vp, vp, i32]),
    "yh_cache_query": (i32, [C.c_char_p, vp]),
    "yh_cache_load": (i32, [C.c_char_p, C.c_uint64, vp, i32, vp, i32, vp, i32, vp, i32, vp, vp, i32]),
}

_lib = None


class YuneError(RuntimeError):
    """A C-ABI call returned a negative status."""

    def __init__(self, code, msg):
        super().__init__("%s (code %d)" % (msg, code))
        self.code = code


def lib():
    """The loaded library; raises ImportError when it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libyune_gb300.so is not built; run: python -c 'import __graft_entry__ as g; g.build()'")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


# status codes of the core (include/yune_cuda.h)
YC_E_INVALID, YC_E_NOMEM, YC_E_LAUNCH, YC_E_TIMEOUT, YC_E_NODEVICE, YC_E_OVERFLOW, YC_E_BUDGET, YC_E_NOTFOUND = \
    -1, -2, -3, -4, -5, -6, -7, -8


def device_allocations():
    """Device allocations the library's contexts and batches have made in this process
    (yc_device_allocations)."""
    n = C.c_uint64()
    check(lib().yc_device_allocations(C.byref(n)), "yc_device_allocations")
    return int(n.value)


# status codes of the host producers (include/yune_host.h)
YH_E_INVALID, YH_E_NOMEM, YH_E_RANGE, YH_E_IO, YH_E_FORMAT, YH_E_STALE = -1, -2, -3, -4, -5, -6
HOST_ERRORS = {YH_E_INVALID: "invalid argument", YH_E_NOMEM: "host allocation failed",
               YH_E_RANGE: "index or size out of range", YH_E_IO: "file cannot be opened, read or written",
               YH_E_FORMAT: "not a scene cache of this format, truncated or corrupt",
               YH_E_STALE: "scene cache made for another key"}


def check_host(rc, what=""):
    """check() for the yh_* host functions, which report by status code alone."""
    if rc != 0:
        raise YuneError(rc, (what + ": " if what else "") + HOST_ERRORS.get(rc, "error"))
    return rc


def check(rc, what=""):
    if rc != 0:
        msg = lib().yc_last_error()
        msg = msg.decode() if msg else ""
        raise YuneError(rc, (what + ": " if what else "") + msg)
    return rc
