"""The C-ABI from plain C: tests/c_abi/consumer.c includes include/yune_cuda.h and
include/yune_host.h, is compiled as C11 with every warning an error, links
libyune_gb300.so and runs the host producers, the BVH refit, the scene cache and image
output through it; yc_create must fail cleanly on a machine without a CUDA device (and
succeed on one with). CPU only: no kernel is launched."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "yune_gb300")


@pytest.mark.skipif(shutil.which("gcc") is None, reason="no C compiler")
def test_c11_consumer(tmp_path):
    exe = str(tmp_path / "consumer")
    cmd = ["gcc", "-std=c11", "-Wall", "-Wextra", "-pedantic", "-Werror", "-O1",
           "-I" + os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "c_abi", "consumer.c"),
           "-L" + LIBDIR, "-lyune_gb300", "-Wl,-rpath," + LIBDIR, "-o", exe]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout
    r = subprocess.run([exe, str(tmp_path)], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                       timeout=120)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stdout
    assert "device:" in r.stdout
