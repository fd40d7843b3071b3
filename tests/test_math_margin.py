"""How far the reference's image moves when its OpenCL built-ins come from another
implementation. The kernels, the oracle and the compiled reference all take cos, sin and
pow from ym_math.h (the bit-parity contract needs one implementation on both sides); the
OpenCL spec leaves their last bits to the runtime. Here the compiled reference is built
a second time with the host C library's cosf, sinf and powf (cl_shim.hpp, YREF_LIBM) and
the two images are compared: the margin the per-pixel 1e-3 contract has against a
runtime whose built-ins round differently. CPU only (the compiled reference)."""
import numpy as np
import pytest

from oracle import oracle_py as O
from yune_gb300 import scenes


@pytest.fixture(scope="module")
def libs():
    if O.ref() is None or O.ref_libm() is None:
        pytest.skip("the reference's kernel text is not available")


def _render(s, variant, rr, max_depth, seeds, libm, stop=None):
    acc = np.zeros((s.height, s.width, 4), np.float32)
    out = {}
    for k, sd in enumerate(seeds):
        O.ref_render(s, acc, sd, 1 if k == 0 else 0, variant, rr, max_depth, libm=libm)
        if stop and k + 1 in stop:
            out[k + 1] = acc[..., :3].astype(np.float64)
    return out


@pytest.mark.parametrize("name", ["c0", "c1_l5"])
def test_udpt_every_pixel_within_1e3_with_libm_builtins(libs, name):
    """Unidirectional paths (the configurations' variant B: MIS, Oren-Nayar, RR 3): after 1
    and 16 passes every pixel of the libm build is within 1e-3 relative of the ym_math
    build (measured: largest difference about 1e-4; 68-94% of pixels bit-equal)."""
    s = scenes.c0(48, 48) if name == "c0" else scenes.c1(48, 48, level=5)
    md = 100000 if name == "c0" else 16
    seeds = scenes.pass_seeds(11, 16)
    a = _render(s, "udpt_mis_on", 3, md, seeds, False, (1, 16))
    b = _render(s, "udpt_mis_on", 3, md, seeds, True, (1, 16))
    for n in (1, 16):
        rel = np.abs(a[n] - b[n]) / np.maximum(np.abs(a[n]), 1e-6)
        assert rel.max() <= 1e-3, (n, rel.max())
    assert not np.array_equal(a[16], b[16])   # the built-ins do differ in their last bits


def test_bdpt_image_within_noise_with_libm_builtins(libs):
    """Naive BDPT (8 vertices per subpath, four lights) is more sensitive: a last-bit
    change of a sampled direction moves connections of many vertices, so per pixel the
    libm image is not within 1e-3 of the ym_math one (measured after 8 passes: 63% of
    pixels are). As images they agree far inside the Monte Carlo noise: the RMSE between
    the two builds is below a tenth of the RMSE between two seed sets (measured 0.014 vs
    0.40 of the mean after 8 passes), and the means agree to 1e-3."""
    s = scenes.c0_bdpt(48, 48, bounces=8, lights=4)
    seeds, other = scenes.pass_seeds(11, 8), scenes.pass_seeds(12, 8)
    a = _render(s, "bdpt8_l4", 3, 100000, seeds, False, (8,))[8]
    b = _render(s, "bdpt8_l4", 3, 100000, seeds, True, (8,))[8]
    c = _render(s, "bdpt8_l4", 3, 100000, other, False, (8,))[8]
    rmse_libm = np.sqrt(((a - b) ** 2).mean())
    rmse_seed = np.sqrt(((a - c) ** 2).mean())
    assert rmse_libm < 0.1 * rmse_seed, (rmse_libm, rmse_seed)
    assert abs(b.mean() / a.mean() - 1.0) < 1e-3
