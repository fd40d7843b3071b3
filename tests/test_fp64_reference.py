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


@pytest.mark.parametrize("name", ["c0_mis", "c0_bdpt_mis"])
def test_bdpt_mis_agrees_with_the_independent_reference(name):
    """The bidirectional tracer with MIS (FP64 CPU statement, 1,024 passes) against the
    65,536-pass image of the same scene made by another estimator, the next-event-only
    unidirectional tracer with the same longest path: the mean error over the 1,024 pixels
    stays within 5 standard errors (a 1% offset would be about 10)."""
    ref = quality.load_reference(name)
    assert ref is not None and ref["n_pass"] == 65536
    s = scenes.CONFIGS[name]()
    seeds = scenes.mt19937(31, 1024)
    px = O.reference_pixels_f64(s, ref["xs"], ref["ys"], seeds, s.cfg, bdpt_bounces=s.cfg["bdpt_bounces"],
                                bdpt_mis=True)
    err = (px[:, :3] - ref["ref"][:, :3]).mean(axis=1)
    assert abs(err.mean()) < 5.0 * err.std() / np.sqrt(len(err))
    assert abs(err.mean()) < 0.004 * ref["ref"][:, :3].mean()


def test_reference_mis_branch_converges_above_next_event_only():
    """A measured property of the reference estimator: udpt.cl's MIS branch of
    evaluateDirectLighting (udpt.cl:570-608; with the lobe fix) converges about 1% above
    the next-event-only tracer on C0 (65,536 passes of each), which the bidirectional
    tracer with MIS matches instead. Its weights use calcPhongPDF (udpt.cl:1033-1045),
    which takes the cosine of a cosine, so the two weights of a glossy sample do not sum
    to one."""
    mis = quality.load_reference("c0")
    nee = quality.load_reference("c0_mis")
    assert np.array_equal(mis["xs"], nee["xs"]) and np.array_equal(mis["ys"], nee["ys"])
    err = (mis["ref"][:, :3] - nee["ref"][:, :3]).mean(axis=1)
    z = err.mean() / (err.std() / np.sqrt(len(err)))
    rel = err.mean() / nee["ref"][:, :3].mean()
    assert z > 5.0 and 0.005 < rel < 0.02


@pytest.mark.parametrize("name", ["c2_j0", "c2_j8", "c2_j16", "c3_s2", "c3_s4"])
def test_mix_and_pool_references_are_unbiased(name):
    """The references of three jobs of the mixed workload and two scenes of the serving
    pool (the benchmark's options: NEE + MIS, Oren-Nayar, roulette after bounce 3, at most
    16 bounces) against 32 independent FP64 passes of the same pixels."""
    import importlib.util
    import os
    spec = importlib.util.spec_from_file_location(
        "make_fp64_refs", os.path.join(os.path.dirname(__file__), "golden", "make_fp64_refs.py"))
    mk = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mk)
    ref = quality.load_reference(name)
    assert ref is not None and ref["n_pass"] == 65536
    s = mk.scene_of(name)
    short = O.reference_pixels_f64(s, ref["xs"], ref["ys"], scenes.mt19937(101, 32), s.cfg)
    err = (short[:, :3] - ref["ref"][:, :3]).mean(axis=1)
    assert abs(err.mean()) < 5.0 * err.std() / np.sqrt(len(err))
