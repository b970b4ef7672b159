"""The integer-pipe FP64 -> FP32 narrowing and FP32 -> FP64 widening of
csrc/fp_conv.cuh (f64_to_f32_rn, f32_to_f64), restated step for step in
numpy integer arithmetic and checked against IEEE round-to-nearest-even
(numpy's float64 -> float32 conversion) on random doubles, exact ties, and
both ends of the FP32 normal range, and against numpy's exact widening.
The device functions run the same integer steps (narrowing: add 2^28 - 1 +
lsb to the 64-bit pattern, funnel shift left by 3, subtract 384 << 23;
widening: shift the exponent and mantissa down 3 bits, add 896 << 20), so
this pins them without a GPU; values outside the normal range take the
hardware conversion there and are excluded here."""
import numpy as np


def narrow_bits(d):
    b = d.view(np.uint64)
    hi = (b >> np.uint64(32)).astype(np.uint32)
    normal = ((hi & np.uint32(0x7FF00000)) - np.uint32(0x38100000)) < np.uint32(0x0FE00000)
    with np.errstate(over="ignore"):
        rb = b + (np.uint64(0x0FFFFFFF) + ((b >> np.uint64(29)) & np.uint64(1)))  # rounding carry
    rhi = (rb >> np.uint64(32)).astype(np.uint32)
    rlo = (rb & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    r = ((rhi << np.uint32(3)) | (rlo >> np.uint32(29))) - np.uint32(0xC0000000)  # funnel shift, bias
    out = r | (hi & np.uint32(0x80000000))
    return out, normal


def widen_bits(f):
    u = f.view(np.uint32)
    a = u & np.uint32(0x7FFFFFFF)
    normal = (a - np.uint32(0x00800000)) < np.uint32(0x7F000000)
    hi = ((a >> np.uint32(3)) + np.uint32(0x38000000)) | (u & np.uint32(0x80000000))
    lo = u << np.uint32(29)
    return (hi.astype(np.uint64) << np.uint64(32)) | lo.astype(np.uint64), normal


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



def test_widening_is_exact():
    rng = np.random.default_rng(7)
    n = 2_000_000
    u = rng.integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32)
    e = rng.integers(1, 255, n).astype(np.uint32)
    u = (u & np.uint32(0x807FFFFF)) | (e << np.uint32(23))
    u = np.concatenate([u, np.array([0x00800000, 0x80800000, 0x7F7FFFFF, 0xFF7FFFFF], np.uint32)])
    f = u.view(np.float32)
    got, normal = widen_bits(f)
    assert normal.all()
    assert np.array_equal(got, f.astype(np.float64).view(np.uint64))
    sp = np.array([0.0, -0.0, 1e-40, np.inf, -np.inf, np.nan], np.float32)
    assert not widen_bits(sp)[1].any()
