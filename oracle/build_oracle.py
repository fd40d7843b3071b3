"""Build recipe for the CPU oracle (oracle/liboracle.so) and the compiled reference
(oracle/_ref/libyune_ref.so).

TEST INFRASTRUCTURE: the outputs are checkers and the CPU baseline, never the product.

* liboracle.so   -- the restatement in oracle/udpt_oracle.hpp (+ bdpt_oracle.hpp), and
                    the bidirectional tracer with MIS (bdpt_mis_oracle.hpp).
* _ref/          -- Yune's own kernel files compiled as C++: the syntax-only transform
                    of oracle/ref/transform.py turns kernels/legacy/udpt.cl, bdpt.cl,
                    udpt-primitives.cl and kernels/post-proc/tonemap.cl into .inc files
                    under oracle/_ref/, and oracle/ref/ref_harness.cpp includes them.
                    When the reference tree is present the reference BVH builder
                    (src/BVH.cpp, src/TriangleCPU.cpp, src/BVHNodeCPU.cpp) is compiled
                    in as well, straight from where it lies. On a host without the
                    reference tree the .inc files made earlier are compiled if present.
Host flags: -O3 -ffp-contract=off (no FMA contraction on any host), no -march.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
REF_SRC = "/root/reference"
REF_OUT = os.path.join(HERE, "_ref")

CXX = os.environ.get("CXX", "g++")
CXXFLAGS = ["-std=c++17", "-O3", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-pthread",
            "-Wno-unused-variable", "-Wno-unused-but-set-variable"]

KERNELS = {
    "udpt.inc": "kernels/legacy/udpt.cl",
    "bdpt.inc": "kernels/legacy/bdpt.cl",
    "primitives.inc": "kernels/legacy/udpt-primitives.cl",
    "tonemap.inc": "kernels/post-proc/tonemap.cl",
}


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


def build_oracle(force=False):
    out = os.path.join(HERE, "liboracle.so")
    srcs = [os.path.join(HERE, f) for f in ("oracle_capi.cpp", "udpt_oracle.hpp", "oracle_math.hpp",
                                              "bdpt_oracle.hpp", "bdpt_mis_oracle.hpp")]
    srcs.append(os.path.join(ROOT, "yune_gb300", "csrc", "ym_math.h"))
    if not force and _newer(out, srcs) and _elf_matches_host(out):
        return out
    _run([CXX] + CXXFLAGS + ["-I" + os.path.join(ROOT, "include"), os.path.join(HERE, "oracle_capi.cpp"),
                              "-o", out])
    return out


def build_ref(force=False):
    """Returns the path of libyune_ref.so, or None when no reference text is at hand."""
    os.makedirs(REF_OUT, exist_ok=True)
    have_tree = os.path.isdir(REF_SRC)
    if have_tree:
        sys.path.insert(0, os.path.join(HERE, "ref"))
        import transform  # noqa: E402
        for inc, cl in KERNELS.items():
            src = os.path.join(REF_SRC, cl)
            dst = os.path.join(REF_OUT, inc)
            if force or not _newer(dst, [src, os.path.join(HERE, "ref", "transform.py")]):
                with open(src, "r", encoding="utf-8", errors="replace") as f:
                    text = f.read()
                with open(dst, "w") as f:
                    f.write(transform.transform(text))
    if not all(os.path.exists(os.path.join(REF_OUT, inc)) for inc in KERNELS):
        return None
    out = os.path.join(REF_OUT, "libyune_ref.so")
    deps = [os.path.join(REF_OUT, inc) for inc in KERNELS]
    deps += [os.path.join(HERE, "ref", f) for f in ("ref_harness.cpp", "cl_shim.hpp")]
    deps.append(os.path.join(ROOT, "yune_gb300", "csrc", "ym_math.h"))
    if not force and _newer(out, deps) and _elf_matches_host(out):
        return out
    cmd = [CXX] + CXXFLAGS + ["-I" + REF_OUT, "-I" + os.path.join(HERE, "ref"),
                              os.path.join(HERE, "ref", "ref_harness.cpp")]
    if have_tree:
        cmd += ["-I" + os.path.join(HERE, "ref", "stub_include"), "-I" + os.path.join(REF_SRC, "include")]
        cmd += [os.path.join(REF_SRC, "src", f) for f in ("BVH.cpp", "TriangleCPU.cpp", "BVHNodeCPU.cpp", "Scene.cpp")]
    else:
        cmd += ["-DYREF_NO_HOST"]
    cmd += ["-o", out]
    _run(cmd)
    return out


if __name__ == "__main__":
    print(build_oracle(force=True))
    print(build_ref(force=True))
