"""Accuracy of the portable FP32 built-ins (yune_gb300/csrc/ym_math.h) against float64
numpy, and known answers of the per-pixel RNG (Wang hash, xorshift32 13/17/5 of
kernels/legacy/udpt.cl:1131-1147). The same routines run on the GPU, where their bit
equality with the CPU is covered by the render parity tests."""
import numpy as np

from oracle import oracle_py as O


def _eval(fn, a, b=None):
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b if b is not None else np.zeros_like(a), np.float32)
    out = np.zeros_like(a)
    assert O.orc().or_ym_eval(fn, a.ctypes.data, b.ctypes.data, out.ctypes.data, len(a)) == 0
    return out


def _ulp_err(got, want):
    want32 = want.astype(np.float32)
    spacing = np.spacing(np.abs(want32)).astype(np.float64)
    return np.abs(got.astype(np.float64) - want) / spacing


def test_sin_cos_ulp():
    rng = np.random.default_rng(0)
    x = np.concatenate([rng.uniform(-7, 7, 200000), rng.uniform(-1000, 1000, 20000),
                        np.linspace(-np.pi, np.pi, 4001)]).astype(np.float32)
    xd = x.astype(np.float64)
    assert _ulp_err(_eval(0, x), np.sin(xd))[np.abs(np.sin(xd)) > 1e-3].max() <= 2.0
    assert _ulp_err(_eval(1, x), np.cos(xd))[np.abs(np.cos(xd)) > 1e-3].max() <= 2.0
    # absolute error near the zeros
    assert np.abs(_eval(0, x) - np.sin(xd)).max() < 2e-7 * max(1.0, np.abs(xd).max() / 16)


def test_exp2_log2_ulp():
    rng = np.random.default_rng(1)
    t = rng.uniform(-120, 120, 200000).astype(np.float32)
    assert _ulp_err(_eval(3, t), np.exp2(t.astype(np.float64))).max() <= 2.0
    x = np.exp(rng.uniform(-80, 80, 200000)).astype(np.float32)
    got = _eval(4, x).astype(np.float64)
    want = np.log2(x.astype(np.float64))
    assert (np.abs(got - want) / np.maximum(np.abs(want), 1.0)).max() < 3e-7


def test_pow_domain_of_the_renderer():
    rng = np.random.default_rng(2)
    # pow(r, 1/(n+1)), pow(c, n), pow(c, 5), pow(x, 1/2.2) with x, c, r in [0, 1]
    x = rng.uniform(0, 1, 200000).astype(np.float32)
    y = np.concatenate([1.0 / (rng.integers(1, 400, 100000) + 1), rng.uniform(0, 400, 100000)]).astype(np.float32)
    got = _eval(2, x, y).astype(np.float64)
    xd, yd = x.astype(np.float64), y.astype(np.float64)
    want = np.power(xd, yd)
    m = want > 1e-30
    # exp2(y * log2 x) in FP32: the error of log2 is amplified by |y log2 x|
    bound = 3e-7 * (1.0 + np.abs(yd * np.log2(np.maximum(xd, 1e-45))))
    assert (np.abs(got - want)[m] / want[m] <= bound[m]).all()


def test_pow_special_cases():
    x = np.array([0.0, -0.0, 1.0, 2.0, -2.0, -2.0, np.inf, 0.5, np.nan, 3.0, 0.0], np.float32)
    y = np.array([2.0, 3.0, np.nan, 0.0, 3.0, 0.5, 2.0, np.inf, 1.0, 1.0, -1.0], np.float32)
    got = _eval(2, x, y)
    with np.errstate(all="ignore"):
        want = np.power(x.astype(np.float64), y.astype(np.float64)).astype(np.float32)
    assert np.array_equal(np.isnan(got), np.isnan(want))
    ok = ~np.isnan(want)
    assert np.array_equal(got[ok], want[ok])


def _wang(s):
    s = ((s ^ 61) ^ (s >> 16)) & 0xFFFFFFFF
    s = (s * 9) & 0xFFFFFFFF
    s = s ^ (s >> 4)
    s = (s * 0x27D4EB2D) & 0xFFFFFFFF
    return s ^ (s >> 15)


def _xs(s):
    s ^= (s << 13) & 0xFFFFFFFF
    s ^= s >> 17
    s ^= (s << 5) & 0xFFFFFFFF
    return s & 0xFFFFFFFF


def test_rng_known_answers():
    L = O.orc()
    rng = np.random.default_rng(4)
    for s in [0, 1, 61, 0xFFFFFFFF, 0x80000000] + [int(v) for v in rng.integers(0, 2 ** 32, 1000)]:
        assert L.or_wang_hash(s) == _wang(s)
        assert L.or_xor_shift(s) == _xs(s)
    assert _wang(0) != 0 and _xs(0) == 0   # why the kernel re-hashes a zero seed (udpt.cl:178-180)
