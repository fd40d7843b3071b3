"""Builds libyune_gb300.so in-tree: the CUDA core (sm_103a) and the host producers.

Every .cu file is compiled by nvcc for `-gencode arch=compute_103a,code=sm_103a` with
`-fmad=false` (no multiply-add contraction, so the FP32 arithmetic is the reference
kernel's operation for operation) and the host code with `-ffp-contract=off` for the
same reason. Translation units compile in parallel; the shared object links the CUDA
runtime statically.
"""
import concurrent.futures as cf
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libyune_gb300.so")

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "--fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off",
                   "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]
CXX_FLAGS = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math,-pthread",
             "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]

CU_SOURCES = ["core/api.cu", "core/trace.cu", "core/udpt.cu", "core/bench_kernels.cu", "core/noalloc.cu", "core/bdpt.cu",
              "core/engine.cu", "core/tail.cu", "core/raysort.cu", "core/bvh_build.cu", "core/bdpt_mis.cu", "core/refit.cu",
              "core/repack_dev.cu"]
CXX_SOURCES = ["core/repack.cpp", "core/serve.cpp", "core/walk_host.cpp", "core/tune.cpp", "host/yh_bvh.cpp", "host/yh_camera.cpp", "host/yh_scene.cpp", "host/yh_image.cpp",
               "host/yh_cache.cpp", "host/yh_threads.cpp"]
HEADERS = ["ym_math.h", "core/yc_scene.h", "core/yc_internal.h", "core/yc_traverse.cuh", "core/yc_shade.cuh",
           "core/yc_repack.h", "core/yc_noalloc.h", "core/yc_bdpt.h", "core/yc_udpt.cuh",
           "core/yc_trace_loop.cuh", "core/yc_engine.h", "core/yc_sah.h", "host/yh_threads.h"]


def _deps():
    out = [os.path.join(CSRC, h) for h in HEADERS]
    out += [os.path.join(ROOT, "include", h) for h in ("yune_types.h", "yune_cuda.h", "yune_host.h")]
    return [p for p in out if os.path.exists(p)]


def _obj(src):
    return os.path.join(BUILD, src.replace("/", "_") + ".o")


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _compile(src, flags):
    obj = _obj(src)
    cmd = [NVCC] + flags + ["-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s" % (src, r.stdout[-6000:]))
    return obj


def build(force=False, jobs=None):
    """Compiles the stale translation units and links the library; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    hdr = _deps()
    todo = []
    for src in CU_SOURCES:
        if force or _stale(_obj(src), [os.path.join(CSRC, src)] + hdr):
            todo.append((src, CU_FLAGS))
    for src in CXX_SOURCES:
        if force or _stale(_obj(src), [os.path.join(CSRC, src)] + hdr):
            todo.append((src, CXX_FLAGS))
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 2)) as ex:
        list(ex.map(lambda a: _compile(*a), todo))
    objs = [_obj(s) for s in CU_SOURCES + CXX_SOURCES]
    if force or todo or _stale(LIB, objs):
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lpthread"]
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stdout[-6000:])
    return LIB


if __name__ == "__main__":
    print(build())
