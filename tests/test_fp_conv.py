"""The integer-pipe FP64 -> FP32 narrowing of csrc/fp_conv.cuh
(f64_to_f32_rn), restated step for step in numpy uint32 arithmetic and
checked against IEEE round-to-nearest-even (numpy's float64 -> float32
conversion) on random doubles, exact ties, and both ends of the FP32 normal
range.  The device function runs the same integer steps (funnel shift left
by 3, subtract 384 << 23, carry of dropped + 2^28 - 1 + lsb), so this pins
its rounding without a GPU; values outside the normal range take the
hardware conversion there and are excluded here."""
import numpy as np


def narrow_bits(d):
    b = d.view(np.uint64)
    hi = (b >> np.uint64(32)).astype(np.uint32)
    lo = (b & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    normal = ((hi & np.uint32(0x7FF00000)) - np.uint32(0x38100000)) < np.uint32(0x0FE00000)
    r = ((hi << np.uint32(3)) | (lo >> np.uint32(29))) - np.uint32(0xC0000000)  # funnel shift, bias
    up = ((lo & np.uint32(0x1FFFFFFF)) + np.uint32(0x0FFFFFFF) + (r & np.uint32(1))) >> np.uint32(29)
    out = (r | (hi & np.uint32(0x80000000))) + up
    return out, normal


def test_narrowing_matches_round_to_nearest_even():
    rng = np.random.default_rng(2024)
    n = 4_000_000
    parts = []
    # random mantissas and signs over the FP32 normal exponent range
    b = rng.integers(0, 2 ** 63, n, dtype=np.uint64) | (rng.integers(0, 2, n, dtype=np.uint64) << np.uint64(63))
    e = rng.integers(897, 1151, n, dtype=np.uint64)
    parts.append((b & np.uint64(0x800FFFFFFFFFFFFF)) | (e << np.uint64(52)))
    # exact ties (dropped bits = 1000...0) and their neighbours
    t = parts[0] & np.uint64(0xFFFFFFFFE0000000)
    parts += [t | np.uint64(0x10000000), t | np.uint64(0x0FFFFFFF), t | np.uint64(0x10000001)]
    # all-ones mantissas (carry into the exponent, to infinity at the top)
    parts.append(parts[0] | np.uint64(0x000FFFFFFFFFFFFF))
    d = np.concatenate(parts).view(np.float64)
    got, normal = narrow_bits(d)
    with np.errstate(over="ignore"):
        want = d.astype(np.float32).view(np.uint32)
    assert normal.all()
    assert np.array_equal(got, want), int(np.count_nonzero(got != want))


def test_range_test_sends_specials_to_the_hardware_path():
    vals = np.array([0.0, -0.0, 1e-40, 2.0 ** -127, 2.0 ** 128, np.inf, -np.inf, np.nan, 2.0 ** -126, 3.0e38])
    _, normal = narrow_bits(vals)
    assert list(normal) == [False, False, False, False, False, False, False, False, True, True]

