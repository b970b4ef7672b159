"""The bulk-flux kernel's FP64 reciprocal, exp, log, square root and
reciprocal square root (csrc/fp64_fast.cuh),
through dccm_fp64_fn_dev, against extended-precision references
(np.longdouble: 80-bit on x86, IEEE quad on Arm).

Bound: 2 units in the last place of the double nearest to the exact value,
over random inputs spanning the fast paths' ranges and the ranges the flux
meets (surface pressure ratios near 1, log-height ratios, Clausius-
Clapeyron exponents), and exact agreement with the library on the inputs
that take the fallback (zero, subnormal, out-of-range, infinite, NaN,
negative).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ULP_BOUND = 2.0


def _run(dccm, torch, fn, x):
    dx = torch.from_numpy(np.ascontiguousarray(x, np.float64)).cuda()
    dy = torch.empty_like(dx)
    dccm.fp64_fn_dev(fn, dx, dy)
    torch.cuda.synchronize()
    return dy.cpu().numpy()


def _ulps(got, exact_ld):
    ref = exact_ld.astype(np.float64)
    err = np.abs(got.astype(np.longdouble) - exact_ld)
    return (err / np.spacing(np.abs(ref)).astype(np.longdouble)).astype(np.float64)


def _inputs(rng, kind):
    n = 1 << 16
    if kind == "rcp":
        mant = rng.uniform(1.0, 2.0, n)
        return np.ldexp(mant, rng.integers(-124, 126, n)) * rng.choice([-1.0, 1.0], n)
    if kind in ("sqrt", "rsqrt"):
        return np.concatenate([np.ldexp(rng.uniform(1.0, 2.0, n // 2), rng.integers(-124, 126, n // 2)),
                               rng.uniform(0.0, 2e3, n // 4), 1.0 + rng.uniform(0, 5, n // 4)])
    if kind == "exp":
        return np.concatenate([rng.uniform(-5, 5, n // 4), rng.uniform(-511, 511, n // 4),
                               rng.uniform(-1e-3, 1e-3, n // 4), rng.uniform(-0.3, 0.1, n // 4)])
    return np.concatenate([np.ldexp(rng.uniform(1.0, 2.0, n // 4), rng.integers(-1021, 1023, n // 4)),
                           rng.uniform(0.5, 1.1, n // 4), 1.0 + rng.uniform(-1e-6, 1e-6, n // 4),
                           rng.uniform(1.0, 1e6, n // 4)])


KINDS = ["rcp", "exp", "log", "sqrt", "rsqrt"]


@pytest.mark.parametrize("kind", KINDS)
def test_fast_fp64_functions_within_two_ulp(dccm, cuda, kind):
    rng = np.random.default_rng(1 + KINDS.index(kind))
    x = _inputs(rng, kind)
    fn = {"rcp": dccm.FP64_RCP, "exp": dccm.FP64_EXP, "log": dccm.FP64_LOG, "sqrt": dccm.FP64_SQRT,
          "rsqrt": dccm.FP64_RSQRT}[kind]
    got = _run(dccm, cuda, fn, x)
    xl = x.astype(np.longdouble)
    exact = {"rcp": lambda: np.longdouble(1) / xl, "exp": lambda: np.exp(xl), "log": lambda: np.log(xl),
             "sqrt": lambda: np.sqrt(xl), "rsqrt": lambda: np.longdouble(1) / np.sqrt(xl)}[kind]()
    u = _ulps(got, exact)
    assert float(u.max()) <= ULP_BOUND, (kind, float(u.max()), x[int(np.argmax(u))])


def test_fallback_inputs_match_the_library(dccm, cuda):
    torch = cuda
    with np.errstate(all="ignore"):
        cases = {
            dccm.FP64_RCP: np.array([0.0, -0.0, 5e-324, 1e-310, 2.0 ** -126, 2.0 ** 127, 1e300, -1e300,
                                     np.inf, -np.inf, np.nan]),
            dccm.FP64_EXP: np.array([512.0, 709.0, 710.0, -745.0, -746.0, -1000.0, 1000.0, np.inf, -np.inf, np.nan]),
            dccm.FP64_LOG: np.array([0.0, -0.0, 5e-324, 1e-310, -1.0, np.inf, -np.inf, np.nan, 1.7e308]),
            dccm.FP64_SQRT: np.array([0.0, -0.0, 5e-324, 1e-310, -1.0, 1e300, np.inf, -np.inf, np.nan]),
        }
        for fn, x in cases.items():
            got = _run(dccm, torch, fn, x)
            xl = x.astype(np.longdouble)
            want = {dccm.FP64_RCP: np.longdouble(1) / xl, dccm.FP64_EXP: np.exp(xl),
                    dccm.FP64_LOG: np.log(xl), dccm.FP64_SQRT: np.sqrt(xl)}[fn].astype(np.float64)
            same = (got == want) | (np.isnan(got) & np.isnan(want))
            close = np.abs(got - want) <= 2 * np.spacing(np.abs(want))
            assert np.all(same | close), (fn, x, got, want)
    # argument checks
    dx = torch.zeros(4, dtype=torch.float64, device="cuda")
    with pytest.raises(dccm.DccmError):
        dccm.fp64_fn_dev(7, dx, dx)
