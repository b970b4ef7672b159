"""The area integral that allocates no device memory.

dccm_area_integral_noalloc_dev exists for callers that cannot call
cudaMalloc, such as a model that has already reserved all of the GPU for
its own allocator.  It keeps its scratch in a fixed array inside the
library.  Here it is called through the C ABI and must
agree with the allocating dccm_area_integral_dev, within the tolerance the
other compensated-sum tests use, on two calls in a row.  The second call is
smaller than the first, so stale partial sums left in the shared array by
the first call would show up.  Sizes beyond its limit must be refused.

This file is named to be collected last, and it passes on its own in a
fresh process as well as after the other tests.
"""
import ctypes
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_N = 1 << 26


def _call(lib, name, f, a, n):
    out = ctypes.c_double(0.0)
    st = getattr(lib, name)(ctypes.c_void_p(f.data_ptr()), ctypes.c_void_p(a.data_ptr()), n,
                            ctypes.byref(out), None)
    return st, out.value


def test_noalloc_matches_allocating_entry_point(dccm, cuda):
    torch = cuda
    lib = dccm.load()
    rng = np.random.default_rng(123)
    sizes = [1_000_003, 70_001]  # second call smaller: stale partials would be read if reused
    for n in sizes:
        f = rng.standard_normal(n) * 300.0 + 5.0
        a = rng.uniform(0.5, 2.0, n) * 1e-4
        df = torch.from_numpy(f).cuda()
        da = torch.from_numpy(a).cuda()
        st0, ref = _call(lib, "dccm_area_integral_dev", df, da, n)
        st1, got = _call(lib, "dccm_area_integral_noalloc_dev", df, da, n)
        assert st0 == 0 and st1 == 0, (st0, st1)
        exact = math.fsum((f * a).tolist())
        assert abs(got - ref) <= 1e-14 * abs(ref), (got, ref)
        assert abs(got - exact) <= 1e-14 * abs(exact), (got, exact)


def test_noalloc_limits(dccm, cuda):
    torch = cuda
    lib = dccm.load()
    x = torch.ones(8, dtype=torch.float64, device="cuda")
    st, _ = _call(lib, "dccm_area_integral_noalloc_dev", x, x, MAX_N + 1)
    assert st == -2  # DCCM_ERR_SHAPE, refused before touching memory
    st, v = _call(lib, "dccm_area_integral_noalloc_dev", x, x, 0)
    assert st == 0 and v == 0.0
    st, v = _call(lib, "dccm_area_integral_noalloc_dev", x, x, 8)
    assert st == 0 and v == 8.0
