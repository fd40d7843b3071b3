"""Image error against a converged FP64 reference.

The references are 65,536-pass FP64 renders of each configuration on a 32 x 32 grid of
its pixels (tests/golden/fp64_<config>.npz: pixel coordinates xs, ys and the RGBA
radiance ref). The error of an accumulator at those pixels is

    rmse      = sqrt(mean over the grid and the RGB channels of (image - ref)^2)
    rel_rmse  = rmse / mean(ref RGB)

Monte Carlo noise falls as 1/sqrt(passes) for an unbiased estimator, so the passes that
reach a target relative RMSE follow from one measurement: passes * (rel_rmse / target)^2.
Paths through the glass sphere and the naive BDPT connections have heavy-tailed pixel
noise (a rare firefly can carry most of the squared error of 1,024 pixels), so a trimmed
RMSE, without the 1% of grid pixels with the largest error, is reported beside it as the
statistic whose decay is checked.
"""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "tests", "golden")


def load_reference(config):
    path = os.path.join(GOLDEN, "fp64_%s.npz" % config)
    if not os.path.exists(path):
        return None
    d = np.load(path)
    return {"xs": d["xs"], "ys": d["ys"], "ref": d["ref"], "n_pass": int(d["n_pass"])}


def error(image, ref):
    """rmse, rel_rmse and mean error of an (H, W, 4) accumulator at the reference's pixels."""
    got = image[ref["ys"], ref["xs"], :3].astype(np.float64)
    want = ref["ref"][:, :3].astype(np.float64)
    rmse = float(np.sqrt(np.mean((got - want) ** 2)))
    return rmse, rmse / float(np.mean(want)), float(np.mean(got - want))


def trimmed_rmse(image, ref, drop=0.01):
    """RMSE over the grid without the `drop` fraction of pixels with the largest error."""
    got = image[ref["ys"], ref["xs"], :3].astype(np.float64)
    want = ref["ref"][:, :3].astype(np.float64)
    per = np.mean((got - want) ** 2, axis=1)
    keep = np.sort(per)[: len(per) - int(np.ceil(drop * len(per)))]
    return float(np.sqrt(np.mean(keep)))


def passes_for(rel_rmse, passes, target=0.01):
    """Passes at which the relative RMSE reaches `target`, from 1/sqrt(passes) decay."""
    return int(np.ceil(passes * (rel_rmse / target) ** 2))


def report(image, config, passes, target=0.01):
    ref = load_reference(config)
    if ref is None:
        return None
    rmse, rel, bias = error(image, ref)
    trim = trimmed_rmse(image, ref)
    return {"reference": "fp64, %d passes, %d pixels" % (ref["n_pass"], len(ref["xs"])), "passes": int(passes),
            "rmse": rmse, "rel_rmse": rel, "mean_error": bias, "rmse_trimmed_1pct": trim,
            "rel_rmse_trimmed_1pct": trim / float(np.mean(ref["ref"][:, :3])),
            "passes_for_%g_rel_rmse" % target: passes_for(rel, passes, target)}
