"""The transforms in SPML's real spectral layout (the drop-in a DCPAM caller
links: xya_wa / wa_xya of SPML's wa_module, called by the dynamics at
atm/dcpam_main_mod.f90:2173-2180), through the C ABI.

SPML stores field-level k's coefficients at wa(l_nm(n, m), k),
l_nm = n(n+1) + m + 1, m = -n..n: Re s_n^m at m >= 0, Im s_n^|m| at m < 0.
Its expansion f = sum s_n^m Pbar_n^m e^{i m lon} (s_n^-m = conj s_n^m) gives
the closed forms checked here for single harmonics:
  m = 0:            f = a Pbar_n^0(mu)
  Re slot, m > 0:   f = 2 a Pbar_n^m(mu) cos(m lon)
  Im slot, m > 0:   f = -2 b Pbar_n^m(mu) sin(m lon)
with Pbar_1^0 = sqrt(3) mu, Pbar_1^1 = sqrt(3/2) cos(lat),
Pbar_2^0 = sqrt(5) (3 mu^2 - 1)/2, Pbar_2^1 = sqrt(15/2) mu cos(lat),
Pbar_2^2 = sqrt(15/8) cos^2(lat).
Tolerances: FP64 1e-13, mixed (BF16 x 3) 1e-6 relative; the permutations
alone are bit-exact.
"""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

N, I, J = 21, 64, 32


def _pbar(n, m, mu):
    c = np.sqrt(1.0 - mu * mu)
    return {(0, 0): np.ones_like(mu), (1, 0): np.sqrt(3.0) * mu, (1, 1): np.sqrt(1.5) * c,
            (2, 0): np.sqrt(5.0) * (3 * mu * mu - 1) / 2, (2, 1): np.sqrt(7.5) * mu * c,
            (2, 2): np.sqrt(15.0 / 8.0) * c * c}[(n, m)]


def _wa_to_spec(dccm, wa, N):
    """Python restatement of the permutation: SPML wa -> m-major complex."""
    B = wa.shape[0]
    spec = np.zeros((B, (N + 1) * (N + 2) // 2), np.complex128)
    k = 0
    for m in range(N + 1):
        for n in range(m, N + 1):
            re = wa[:, dccm.l_nm(n, m) - 1]
            im = wa[:, dccm.l_nm(n, -m) - 1] if m > 0 else 0.0
            spec[:, k] = re + 1j * im
            k += 1
    return spec


@pytest.mark.parametrize("prec,tol", [(0, 1e-13), (1, 1e-6)])
def test_single_harmonics_closed_forms(dccm, cuda, prec, tol):
    plan = dccm.ShtPlan(N, I, J, prec, max_batch=16)
    lon, lat, _, _ = plan.axes()
    mu = np.sin(lat)[:, None]
    cases = [(0, 0, 1.0), (1, 0, 0.7), (1, 1, 0.5), (1, -1, -0.3), (2, 0, 1.5), (2, 1, 0.25), (2, -1, 0.8),
             (2, 2, -0.6), (2, -2, 0.4)]
    wa = np.zeros((len(cases), plan.nwa))
    want = np.zeros((len(cases), J, I))
    for b, (n, m, a) in enumerate(cases):
        wa[b, dccm.l_nm(n, m) - 1] = a
        p = _pbar(n, abs(m), mu)
        if m == 0:
            want[b] = a * p * np.ones((1, I))
        elif m > 0:
            want[b] = 2 * a * p * np.cos(m * lon)[None, :]
        else:
            want[b] = -2 * a * p * np.sin(-m * lon)[None, :]
    got = plan.xya_wa(wa)
    for b in range(len(cases)):
        assert rel_l2(got[b], want[b]) <= tol, cases[b]
    # and back: wa_xya of the closed forms recovers the single coefficient
    back = plan.wa_xya(want)
    assert rel_l2(back, wa) <= tol
    assert plan.status() == (0, 0)


@pytest.mark.parametrize("prec,tol", [(0, 1e-13), (1, 1e-6)])
def test_wa_matches_native_layout_and_round_trips(dccm, oracle, synth, cuda, prec, tol):
    torch = cuda
    B = 12
    plan = dccm.ShtPlan(N, I, J, prec, max_batch=B)
    spec = synth.spectra(N, B, seed=3)
    # SPML layout of the same coefficients (Python restatement)
    wa = np.zeros((B, plan.nwa))
    n_, m_ = dccm.nm_l(np.arange(1, plan.nwa + 1))
    k = {}
    kk = 0
    for m in range(N + 1):
        for n in range(m, N + 1):
            k[(n, m)] = kk
            kk += 1
    for l, (n, m) in enumerate(zip(n_, m_)):
        c = spec[:, k[(int(n), abs(int(m)))]]
        wa[:, l] = c.real if m >= 0 else c.imag
    assert np.array_equal(_wa_to_spec(dccm, wa, N), spec)
    go = oracle.sht_inverse(N, I, J, spec)
    # host entry points
    g = plan.xya_wa(wa)
    assert rel_l2(g, go) <= tol
    assert rel_l2(plan.wa_xya(g), wa) <= tol
    # device entry points, and the permutations alone (bit-exact)
    dwa = torch.from_numpy(wa).cuda()
    dg = torch.empty((B, J, I), dtype=torch.float64, device="cuda")
    dwa2 = torch.full_like(dwa, np.nan)
    plan.xya_wa_dev(dwa, dg, B)
    plan.wa_xya_dev(dg, dwa2, B)
    torch.cuda.synchronize()
    assert rel_l2(dg.cpu().numpy(), go) <= tol
    assert rel_l2(dwa2.cpu().numpy(), wa) <= tol
    ds = torch.full((B, spec.shape[1] * 2), np.nan, dtype=torch.float64, device="cuda")
    plan.spec_from_wa_dev(dwa, ds, B)
    torch.cuda.synchronize()
    assert np.array_equal(ds.cpu().numpy().view(np.complex128), spec)
    dwa3 = torch.full_like(dwa, np.nan)
    plan.wa_from_spec_dev(ds, dwa3, B)
    torch.cuda.synchronize()
    assert np.array_equal(dwa3.cpu().numpy(), wa)
    # fewer field-levels than the plan holds; zero is a no-op
    plan.xya_wa_dev(dwa, dg, 5)
    plan.xya_wa_dev(dwa, dg, 0)
    torch.cuda.synchronize()
    assert rel_l2(dg[:5].cpu().numpy(), go[:5]) <= tol
    assert plan.status() == (0, 0)
    with pytest.raises(dccm.DccmError) as e:
        plan.xya_wa_dev(dwa, dg, B + 1)
    assert e.value.status == -2
