"""Converged FP64 references for the RMSE of each configuration.

65,536 passes of the double-precision restatement of the reference kernels
(oracle/udpt_oracle.hpp, oracle/bdpt_oracle.hpp) on a 32 x 32 grid of pixels of each
configuration's frame, with pass seeds from mt19937(7777) (independent of the seeds the
benchmark renders with). Writes tests/golden/fp64_<config>.npz. Runs on the CPU
(FP64_THREADS limits the host threads):

    python tests/golden/make_fp64_refs.py [config ...]
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle_py as O  # noqa: E402
from yune_gb300 import scenes  # noqa: E402

N_PASS = 65536
GRID = 32

# The configurations of the bidirectional tracer with MIS are checked against another
# estimator of the same image: the unidirectional tracer with next-event estimation only
# (udpt.cl with MIS off), its loop bounded so that its paths have the same longest length
# (max_depth = segments - 2).
INDEPENDENT = {"c0_mis": dict(integrator=0, mis=0, max_depth=18),
               "c0_bdpt_mis": dict(integrator=0, mis=0, max_depth=6)}


def grid(s):
    xs = (np.arange(GRID) * s.width) // GRID + s.width // (2 * GRID)
    ys = (np.arange(GRID) * s.height) // GRID + s.height // (2 * GRID)
    X, Y = np.meshgrid(xs, ys)
    return X.ravel().astype(np.int32), Y.ravel().astype(np.int32)


# Scenes of the mixed workload (c2: jobs 0, 8 and 16 of the 64, at their own frame sizes)
# and of the serving pool (c3: scenes 2 and 4 of the 8, at 512 x 512), with the options the
# benchmark renders them with (NEE + MIS, Oren-Nayar, roulette after bounce 3, at most 16
# bounces, the reference's MIS arithmetic).
MIX = {"c2_j0": ("c2", 0), "c2_j8": ("c2", 8), "c2_j16": ("c2", 16), "c3_s2": ("c3", 2), "c3_s4": ("c3", 4)}


def mix_scene(name):
    from yune_gb300 import workloads
    kind, k = MIX[name]
    cfg = scenes.default_cfg(max_depth=16, mis_lobe_fix=0)
    if kind == "c2":
        return workloads.c2_jobs(only=[k], cfg=cfg)[0]
    return workloads.c3_scenes(only=[k], cfg=cfg, width=512, height=512)[0]


def scene_of(name):
    return mix_scene(name) if name in MIX else scenes.CONFIGS[name]()


def make(name, threads=0):
    s = scene_of(name)
    if name in INDEPENDENT:
        s.cfg = dict(s.cfg, **INDEPENDENT[name])
    X, Y = grid(s)
    seeds = scenes.mt19937(7777, N_PASS)
    bounces = s.cfg["bdpt_bounces"] if s.cfg.get("integrator", 0) == 1 else 0
    t0 = time.time()
    ref = O.reference_pixels_f64(s, X, Y, seeds, s.cfg, bdpt_bounces=bounces, threads=threads)
    np.savez_compressed(os.path.join(HERE, "fp64_%s.npz" % name), xs=X, ys=Y, ref=ref, n_pass=N_PASS,
                        seconds=time.time() - t0)
    print(name, "done in %.0f s" % (time.time() - t0))


if __name__ == "__main__":
    threads = int(os.environ.get("FP64_THREADS", "0"))
    for name in (sys.argv[1:] or ["c0", "c1", "c0_bdpt", "c0_mis", "c0_bdpt_mis"] + list(MIX)):
        make(name, threads)
