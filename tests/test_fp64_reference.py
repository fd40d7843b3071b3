"""The converged FP64 references against independent low-pass FP64 renders of the same
pixels: an unbiased reference leaves only zero-mean noise, so the mean error over the
1,024 pixels stays within a few standard errors and the RMSE falls as 1/sqrt(passes)."""
import numpy as np
import pytest

from oracle import oracle_py as O
from yune_gb300 import quality, scenes


@pytest.mark.parametrize("name", ["c0", "c0_bdpt", "c1"])
def test_reference_is_unbiased_against_short_renders(name):
    ref = quality.load_reference(name)
    assert ref is not None and ref["n_pass"] == 65536
    s = scenes.CONFIGS[name]()
    bounces = s.cfg["bdpt_bounces"] if s.cfg.get("integrator", 0) == 1 else 0
    seeds = scenes.mt19937(99, 32)
    img = np.zeros((s.height, s.width, 4), np.float32)
    short = O.reference_pixels_f64(s, ref["xs"], ref["ys"], seeds, s.cfg, bdpt_bounces=bounces)
    img[ref["ys"], ref["xs"]] = short
    rmse, rel, bias = quality.error(img, ref)
    assert rmse > 0.0
    # pixel errors are independent: the mean of 1,024 of them is within 5 standard errors
    err = (short[:, :3] - ref["ref"][:, :3]).mean(axis=1)
    assert abs(err.mean()) < 5.0 * err.std() / np.sqrt(len(err))
    assert abs(bias) < 5.0 * rmse / np.sqrt(len(ref["xs"]))


def test_passes_for_target_follows_inverse_sqrt():
    assert quality.passes_for(0.02, 100, 0.01) == 400
    assert quality.passes_for(0.01, 256, 0.01) == 256


@pytest.mark.parametrize("name", ["c0_bdpt", "c1"])
def test_trimmed_error_halves_when_passes_quadruple(name):
    """Heavy-tailed configurations: without the 1% firefly pixels the error decays as
    1/sqrt(passes) towards the reference, i.e. the reference has no offset."""
    ref = quality.load_reference(name)
    s = scenes.CONFIGS[name]()
    bounces = s.cfg["bdpt_bounces"] if s.cfg.get("integrator", 0) == 1 else 0
    seeds = scenes.mt19937(6, 256)
    trims = []
    for n in (64, 256):
        px = O.reference_pixels_f64(s, ref["xs"], ref["ys"], seeds[:n], s.cfg, bdpt_bounces=bounces)
        img = np.zeros((s.height, s.width, 4))
        img[ref["ys"], ref["xs"]] = px
        trims.append(quality.trimmed_rmse(img, ref))
    assert 1.6 < trims[0] / trims[1] < 2.4
