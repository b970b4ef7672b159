"""GPU parity of the implicit surface coupling sweeps against the FP64
oracle, through the C ABI.  Tolerance: every finite value within 1e-13 of
the array's largest magnitude (the GPU multiplies by shared reciprocals
where the reference divides); the level-1 values the reference divides by
its zero sub-diagonal must be the same infinities (with sign) or NaN."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

TOL = 1e-13


def _close(a, o, name):
    fin = np.isfinite(o)
    assert np.array_equal(np.isfinite(a), fin), name
    assert np.array_equal(np.isnan(a), np.isnan(o)), name
    assert np.array_equal(np.signbit(a[~fin & ~np.isnan(o)]), np.signbit(o[~fin & ~np.isnan(o)])), name
    scale = np.abs(o[fin]).max()
    assert np.abs(a[fin] - o[fin]).max() <= TOL * scale, (name, np.abs(a[fin] - o[fin]).max() / scale)


@pytest.mark.parametrize("ncol,kmax,ncmax", [(24, 12, 2), (32768, 32, 1), (1000, 48, 3)])
def test_forward_matches_oracle(dccm, oracle, synth, ncol, kmax, ncmax):
    d = synth.column_profiles(ncol, kmax, ncmax=ncmax, seed=kmax)
    ih2o = ncmax  # the vapour tracer need not be the first
    o = oracle.implcpl_forward(d, ih2o, synth.IMPLCPL_CONSTS)
    plan = dccm.ImplCplPlan(ncol, kmax, ncmax, ih2o, synth.IMPLCPL_CONSTS)
    g = plan.forward(d)
    for k in ("DUDt", "DVDt", "DTempDt", "DQMixDt", "ImplCplCoef1", "ImplCplCoef2"):
        _close(g[k], o[k], k)
    m = plan.matrices()
    for k in ("UVMtx", "TempMtx", "QMixMtx"):
        _close(m[k], o[k], k)


def test_golden_fixture(dccm):
    z = np.load(os.path.join(GOLDEN, "implcpl_small.npz"))
    d = {k[3:]: z[k] for k in z.files if k.startswith("in_")}
    ncmax, kmax1, ncol = d["QMixFlux"].shape
    plan = dccm.ImplCplPlan(ncol, kmax1 - 1, ncmax, int(z["ih2o"]), z["consts"])
    g = plan.forward(d)
    for k in ("DUDt", "DVDt", "DTempDt", "DQMixDt", "ImplCplCoef1", "ImplCplCoef2"):
        _close(g[k], z["out_" + k], k)


def test_backward_matches_oracle(dccm, oracle, synth, cuda):
    """The coupler's cycle: forward, the surface values at level 1, backward
    (host and device entry points give the same bits)."""
    torch = cuda
    ncol, kmax, ncmax = 8192, 26, 2
    d = synth.column_profiles(ncol, kmax, ncmax=ncmax, seed=4)
    o = oracle.implcpl_forward(d, 1, synth.IMPLCPL_CONSTS)
    plan = dccm.ImplCplPlan(ncol, kmax, ncmax, 1, synth.IMPLCPL_CONSTS)
    g = plan.forward(d)
    rng = np.random.Generator(np.random.PCG64(1))
    lev1 = {k: rng.normal(0, 1e-3, ncol) for k in ("DUDt", "DVDt", "DTempDt")}
    qlev1 = rng.normal(0, 1e-7, (ncmax, ncol))
    for t in (o, g):
        for k, v in lev1.items():
            t[k][0] = v
        t["DQMixDt"][:, 0] = qlev1
    ob = oracle.implcpl_backward(o, o, synth.IMPLCPL_CONSTS[3])
    hb = {k: np.ascontiguousarray(g[k]) for k in ("DUDt", "DVDt", "DTempDt", "DQMixDt")}
    dv = {k: torch.from_numpy(v.copy()).cuda() for k, v in hb.items()}
    plan.backward(hb)
    plan.backward_dev(dv)
    torch.cuda.synchronize()
    for k in hb:
        _close(hb[k], ob[k], k)
        assert np.array_equal(dv[k].cpu().numpy(), hb[k]), k


def test_device_entry_matches_host_entry(dccm, synth, cuda):
    torch = cuda
    ncol, kmax = 4096, 16
    d = synth.column_profiles(ncol, kmax, ncmax=1, seed=2)
    plan = dccm.ImplCplPlan(ncol, kmax, 1, 1, synth.IMPLCPL_CONSTS)
    h = plan.forward(d)
    dd = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in d.items()}
    out = {k: torch.empty(v.shape, dtype=torch.float64, device="cuda") for k, v in h.items()}
    plan.forward_dev(dd, out)
    torch.cuda.synchronize()
    for k, v in h.items():
        got = out[k].cpu().numpy()
        assert np.array_equal(np.isfinite(got), np.isfinite(v)), k
        assert np.array_equal(got[np.isfinite(v)], v[np.isfinite(v)]), k


def test_invalid_arguments(dccm):
    for args in [(10, 1, 1, 1), (10, 8, 1, 2), (0, 8, 1, 1), (10, 8, 2, 0)]:
        with pytest.raises(dccm.DccmError) as e:
            dccm.ImplCplPlan(*args)
        assert e.value.status == -1  # DCCM_ERR_INVALID_ARG
