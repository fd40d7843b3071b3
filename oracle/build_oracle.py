"""Build recipe for the CPU oracle (oracle/liboracle.so) and the compiled reference
(oracle/_ref/libyune_ref.so).

TEST INFRASTRUCTURE: the outputs are checkers and the CPU baseline, never the product.

* liboracle.so   -- the restatement in oracle/udpt_oracle.hpp (+ bdpt_oracle.hpp), and
                    the bidirectional tracer with MIS (bdpt_mis_oracle.hpp); plus the
                    procedural scene producers (yh_scene.cpp, yh_camera.cpp), the inputs
                    of the CPU baseline.
* _ref/          -- Yune's own kernel files compiled as C++: the syntax-only transform
                    of oracle/ref/transform.py turns kernels/legacy/udpt.cl, bdpt.cl,
                    udpt-primitives.cl and kernels/post-proc/tonemap.cl into .inc files
                    under oracle/_ref/ (plus udpt_on.inc, udpt.cl with the Oren-Nayar
                    rule of udpt-primitives.cl grafted in, transform.graft_oren_nayar),
                    and oracle/ref/ref_harness.cpp includes them. The reference's host
                    code (src/BVH.cpp, src/TriangleCPU.cpp, src/BVHNodeCPU.cpp, src/Scene.cpp
                    and the headers of include/) is staged unchanged into oracle/_ref/host/
                    and compiled in from there, so a host without the reference tree (the
                    GPU machine) builds the same library from what was staged.
Host flags: -O3 -ffp-contract=off (no FMA contraction on any host), no -march.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
REF_OUT = os.path.join(HERE, "_ref")


def reference_tree():
    """Directory of the Yune checkout the compiled reference is built from: the
    YUNE_REFERENCE_TREE environment variable, else a checkout named `reference` beside
    this repository's directory. None when neither exists (the .inc files made earlier,
    if any, are then compiled without the host sources)."""
    env = os.environ.get("YUNE_REFERENCE_TREE")
    if env:
        return env if os.path.isdir(env) else None
    beside = os.path.join(os.path.dirname(ROOT), "reference")
    return beside if os.path.isdir(os.path.join(beside, "kernels", "legacy")) else None

CXX = os.environ.get("CXX", "g++")
CXXFLAGS = ["-std=c++17", "-O3", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-pthread",
            "-Wno-unused-variable", "-Wno-unused-but-set-variable"]

KERNELS = {
    "udpt.inc": "kernels/legacy/udpt.cl",
    "bdpt.inc": "kernels/legacy/bdpt.cl",
    "primitives.inc": "kernels/legacy/udpt-primitives.cl",
    "tonemap.inc": "kernels/post-proc/tonemap.cl",
}
# udpt.cl with udpt-primitives.cl's Oren-Nayar diffuse rule (the configurations' variant B)
GRAFTS = {"udpt_on.inc": ("kernels/legacy/udpt.cl", "kernels/legacy/udpt-primitives.cl")}
HOST_SOURCES = ("src/BVH.cpp", "src/TriangleCPU.cpp", "src/BVHNodeCPU.cpp", "src/Scene.cpp")
HOST_DIR = os.path.join(REF_OUT, "host")


def _newer(out, deps):
    if not os.path.exists(out):
        return False
    t = os.path.getmtime(out)
    return all(os.path.getmtime(d) <= t for d in deps if os.path.exists(d))


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: " + " ".join(cmd) + "\n" + r.stdout[-4000:])
    return r.stdout


def _elf_matches_host(path):
    """True when the shared object was built for this machine's architecture."""
    import platform
    try:
        with open(path, "rb") as f:
            hdr = f.read(20)
    except OSError:
        return False
    if len(hdr) < 20 or hdr[:4] != b"\x7fELF":
        return False
    machine = int.from_bytes(hdr[18:20], "little")
    want = {"x86_64": 62, "aarch64": 183, "arm64": 183}.get(platform.machine())
    return want is None or machine == want


# The procedural scene producers (the benchmark's input generator), compiled into the
# oracle library as well so that the CPU baseline makes the same inputs without loading
# the product library.
SCENE_SOURCES = [os.path.join(ROOT, "yune_gb300", "csrc", "host", f) for f in ("yh_scene.cpp", "yh_camera.cpp")]


def build_oracle(force=False):
    out = os.path.join(HERE, "liboracle.so")
    srcs = [os.path.join(HERE, f) for f in ("oracle_capi.cpp", "udpt_oracle.hpp", "oracle_math.hpp",
                                              "bdpt_oracle.hpp", "bdpt_mis_oracle.hpp")]
    srcs.append(os.path.join(ROOT, "yune_gb300", "csrc", "ym_math.h"))
    srcs += SCENE_SOURCES
    if not force and _newer(out, srcs) and _elf_matches_host(out):
        return out
    _run([CXX] + CXXFLAGS + ["-I" + os.path.join(ROOT, "include"), os.path.join(HERE, "oracle_capi.cpp")] +
         SCENE_SOURCES + ["-o", out])
    return out


def build_ref(force=False, libm=False):
    """Returns the path of libyune_ref.so, or None when no reference text is at hand. With
    libm, libyune_ref_libm.so: the same kernels with the host C library's cosf, sinf and
    powf as the OpenCL built-ins (cl_shim.hpp, YREF_LIBM)."""
    os.makedirs(REF_OUT, exist_ok=True)
    REF_SRC = reference_tree()
    have_tree = REF_SRC is not None
    if have_tree:
        sys.path.insert(0, os.path.join(HERE, "ref"))
        import transform  # noqa: E402
        tf = os.path.join(HERE, "ref", "transform.py")

        def read(rel):
            with open(os.path.join(REF_SRC, rel), "r", encoding="utf-8", errors="replace") as f:
                return f.read()
        for inc, cl in KERNELS.items():
            dst = os.path.join(REF_OUT, inc)
            if force or not _newer(dst, [os.path.join(REF_SRC, cl), tf]):
                with open(dst, "w") as f:
                    f.write(transform.transform(read(cl)))
        for inc, (cl, prim) in GRAFTS.items():
            dst = os.path.join(REF_OUT, inc)
            if force or not _newer(dst, [os.path.join(REF_SRC, cl), os.path.join(REF_SRC, prim), tf]):
                with open(dst, "w") as f:
                    f.write(transform.transform(transform.graft_oren_nayar(read(cl), read(prim))))
        # stage the host sources and headers unchanged (a build without the tree uses them)
        import shutil
        os.makedirs(os.path.join(HOST_DIR, "src"), exist_ok=True)
        os.makedirs(os.path.join(HOST_DIR, "include"), exist_ok=True)
        for rel in HOST_SOURCES:
            shutil.copy2(os.path.join(REF_SRC, rel), os.path.join(HOST_DIR, rel))
        for h in os.listdir(os.path.join(REF_SRC, "include")):
            if h.endswith(".h"):
                shutil.copy2(os.path.join(REF_SRC, "include", h), os.path.join(HOST_DIR, "include", h))
    incs = list(KERNELS) + list(GRAFTS)
    if not all(os.path.exists(os.path.join(REF_OUT, inc)) for inc in incs):
        return None
    have_host = all(os.path.exists(os.path.join(HOST_DIR, rel)) for rel in HOST_SOURCES)
    out = os.path.join(REF_OUT, "libyune_ref_libm.so" if libm else "libyune_ref.so")
    deps = [os.path.join(REF_OUT, inc) for inc in incs]
    if have_host:
        deps += [os.path.join(HOST_DIR, rel) for rel in HOST_SOURCES]
    deps += [os.path.join(HERE, "ref", f) for f in ("ref_harness.cpp", "cl_shim.hpp")]
    deps.append(os.path.join(ROOT, "yune_gb300", "csrc", "ym_math.h"))
    if not force and _newer(out, deps) and _elf_matches_host(out):
        return out
    cmd = [CXX] + CXXFLAGS + ["-I" + REF_OUT, "-I" + os.path.join(HERE, "ref"),
                              os.path.join(HERE, "ref", "ref_harness.cpp")]
    if have_host:
        cmd += ["-I" + os.path.join(HERE, "ref", "stub_include"), "-I" + os.path.join(HOST_DIR, "include")]
        cmd += [os.path.join(HOST_DIR, rel) for rel in HOST_SOURCES]
    else:
        cmd += ["-DYREF_NO_HOST"]
    if libm:
        cmd += ["-DYREF_LIBM"]
    cmd += ["-o", out]
    _run(cmd)
    return out


if __name__ == "__main__":
    print(build_oracle(force=True))
    print(build_ref(force=True))
