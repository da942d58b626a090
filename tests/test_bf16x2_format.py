"""The BF16 hi+lo value storage, on the CPU: the oracle's restatement of the
format keeps every value within 2^-23 |hi| of it before decoding and
within (2^-23 + 2^-24) |v| after the kernels' one-fma decode, hi alone is bf16(v), and
the special cases (zero, ties, the BF16 overflow threshold, subnormals,
infinities) come out as the format says."""
import numpy as np

import oracle


def _parts(w):
    w = np.asarray(w, np.uint32)
    hi = (w & np.uint32(0xFFFF0000)).view(np.float32).astype(np.float64)
    d = (w & np.uint32(0xFFFF)).astype(np.uint16).view(np.int16).astype(np.int64)
    return hi, d


def test_error_bounds_over_magnitudes():
    rng = np.random.default_rng(3)
    v = rng.standard_normal(400_000) * np.exp(rng.uniform(-60, 60, 400_000))
    w = oracle.bf16x2_split(v)
    hi, d = _parts(w)
    assert np.all(np.abs(hi - v) <= 2.0 ** -8 * np.abs(v))        # hi: 8 significant bits, nearest
    assert np.all(np.abs(d) <= 16448)                            # |v - hi| <= 2^-8 |hi|: 15 bits of d
    stored = hi * (1.0 + d * 2.0 ** -22)
    assert np.all(np.abs(stored - v) <= 2.0 ** -23 * np.abs(hi))
    dec = oracle.bf16x2_value(w).astype(np.float64)
    assert np.all(np.abs(dec - v) <= (2.0 ** -23 + 2.0 ** -24) * np.abs(v))
    # far tighter than a BF16 low half: normwise error of a random vector
    assert np.linalg.norm(dec - v) / np.linalg.norm(v) < 1.5e-7


def test_hi_is_round_to_nearest_even_bf16():
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: even (1.0) wins
    cases = {1.0: 0x3F80, 1 + 2.0 ** -8: 0x3F80, 1 + 3 * 2.0 ** -8: 0x3F82, -2.5: 0xC020,
             1 + 2.0 ** -8 + 2.0 ** -40: 0x3F81}
    for v, hb in cases.items():
        w = int(oracle.bf16x2_split(np.array([v]))[0])
        assert w >> 16 == hb, (v, hex(w))


def test_special_values():
    v = np.array([0.0, -0.0, np.inf, -np.inf, 3.4e38, 1e-40, 2.0 ** -101, 2.0 ** -99])
    hi, d = _parts(oracle.bf16x2_split(v))
    assert hi[0] == 0 and d[0] == 0 and hi[1] == 0 and d[1] == 0
    assert np.isinf(hi[2]) and np.isinf(hi[3]) and d[2] == 0 and d[3] == 0
    assert np.isinf(hi[4]) and d[4] == 0           # past the BF16 overflow threshold
    assert hi[5] == 2.0 ** -133 and d[5] == 0      # BF16 subnormal, no correction below 2^-100
    assert hi[6] == 2.0 ** -101 and d[6] == 0
    assert hi[7] == 2.0 ** -99
