"""The FP32 sweep's fixed-point FSR tally, restated in numpy on CPU.

A work unit's tally adds contributions x (already multiplied by the unit's
power-of-two scale, so |x| < 2^50 / max_hits) as a signed high word counting
2^20 and an unsigned low word: for |x| >= 2^23 (an integer in FP32),
hi = floor(x / 2^20) and lo = x - hi * 2^20 in [0, 2^20); smaller x go to an
FP32 side sum. This checks, with 32-bit wrap-around words as on the device,
that max_hits adds of extreme contributions neither overflow a word nor lose
a bit, and that the power-of-two scale keeps |x| inside the range."""
import numpy as np

MAX_HITS = 2048  # the layout builder rejects work units above this


def split(xs):
    """The device split: FP32 floor, then the remainder (exact: xs is an
    integer-valued FP32 number, so an FMA gives it without rounding, as the
    FP64 arithmetic here does) and 32-bit conversions."""
    xs = np.float32(xs)
    hf = np.floor(np.float32(xs * np.float32(2.0 ** -20)))
    hi = np.int32(hf)
    rem = np.float64(xs) - np.float64(hf) * 2.0 ** 20
    assert rem == np.float32(rem) and 0 <= rem < 2 ** 20
    return hi, np.uint32(np.int32(np.float32(rem)))


def accumulate(values):
    hi_w, lo_w, small = np.int32(0), np.uint32(0), np.float32(0)
    with np.errstate(over="ignore"):
        for x in values:
            if abs(np.float32(x)) >= np.float32(2.0 ** 23):
                hi, lo = split(x)
                hi_w = np.int32(hi_w + hi)      # wraps like the device word
                lo_w = np.uint32(lo_w + lo)
            elif x != 0:
                small = np.float32(small + np.float32(x))
    return int(hi_w) * 2 ** 20 + int(lo_w), small


def fixed_scale(m, sum_w, hits):
    """The device's unit scale: 2^(50 - E) with bound < 2^E."""
    bound = np.float32(2.0) * np.float32(m) * np.float32(sum_w) * np.float32(hits)
    e = int(((np.float32(bound).view(np.uint32) >> 23) & 0xFF)) - 126
    se = max(-126, min(100, 50 - e))
    return 2.0 ** se


def test_extreme_contributions_do_not_overflow():
    rng = np.random.default_rng(3)
    for sign in (1.0, -1.0, None):
        limit = 2.0 ** 50 / MAX_HITS
        if sign is None:
            vals = rng.uniform(-limit, limit, MAX_HITS)
        else:
            vals = np.full(MAX_HITS, sign * np.nextafter(np.float32(limit), np.float32(0)))
        vals = vals.astype(np.float32)
        fixed, small = accumulate(vals)
        exact = sum(int(v) for v in vals if abs(v) >= 2.0 ** 23)
        assert fixed == exact
        assert small == 0


def test_small_contributions_keep_fp32_precision():
    vals = np.float32([3.0e7, 1.5e-3, -2.0e-4, 9.0e6, 4.0e-5])
    fixed, small = accumulate(vals)
    assert fixed == int(np.float32(3.0e7)) + int(np.float32(9.0e6))
    assert abs(small - np.float32(1.5e-3 - 2.0e-4 + 4.0e-5)) < 1e-9


def test_unit_scale_bounds_every_contribution():
    rng = np.random.default_rng(7)
    for _ in range(200):
        m = 10.0 ** rng.uniform(-20, 10)
        sum_w = 10.0 ** rng.uniform(-3, 1)
        hits = int(rng.integers(1, MAX_HITS + 1))
        scale = fixed_scale(m, sum_w, hits)
        # the largest contribution of the unit, 2 m sum_w, times the scale
        assert 2.0 * m * sum_w * scale < 2.0 ** 50 / hits
        # and the scale is not needlessly small (within a factor 4 of the
        # limit) unless it sits at its cap of 2^100, where a unit's fluxes are
        # so small that its contributions take the FP32 side path
        if scale < 2.0 ** 100:
            assert 2.0 * m * sum_w * scale * hits >= 2.0 ** 47
