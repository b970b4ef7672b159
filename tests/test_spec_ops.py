"""Spectral-space operators (Laplacian, inverse Laplacian, hyperdiffusion
tendency and implicit step) per total wavenumber n.  The reference's code
for them is external (dcpam5), so parity is unpinned: the oracle is
checked against the mathematics' known answers on CPU, and the GPU
against the oracle (relative 1e-14 of the largest coefficient)."""
import os

import numpy as np
import pytest

A = 6.371e6       # planet radius (m)
TAU = 3 * 3600.0  # e-folding time of the largest wavenumber, HDEFoldTimeValue = 3 hour
DT = 1200.0


def nvals(N):
    return np.concatenate([np.arange(m, N + 1) for m in range(N + 1)])


def test_oracle_known_answers(oracle, synth):
    N = 21
    s = synth.spectra(N, 3, seed=5)
    s[:, 0] = 1.0 + 0.5j
    n = nvals(N)
    lap = oracle.spec_apply(N, oracle.SPEC_LAPLACIAN, s, A)
    assert np.allclose(lap, -n * (n + 1) / A ** 2 * s, rtol=1e-15, atol=0)
    back = oracle.spec_apply(N, oracle.SPEC_INV_LAPLACIAN, lap, A)
    assert np.allclose(back[:, 1:], s[:, 1:], rtol=1e-14, atol=0) and np.all(back[:, 0] == 0)
    one = np.ones((1, len(n)), np.complex128)
    for corr in (False, True):
        ten = oracle.spec_apply(N, oracle.SPEC_HDIFF_TENDENCY, one, A, 8, TAU, 0.0, corr)[0].real
        imp = oracle.spec_apply(N, oracle.SPEC_HDIFF_IMPLICIT, one, A, 8, TAU, TAU, corr)[0].real
        top = n == N
        assert np.allclose(ten[top], -1.0 / TAU, rtol=1e-14)       # wavenumber N decays by e in tau
        assert np.allclose(imp[top], 0.5, rtol=1e-14)             # 1 / (1 + tau / tau)
        assert np.allclose(imp, 1.0 / (1.0 - TAU * ten), rtol=1e-14)
        assert np.all(np.diff(ten[n.argsort(kind="stable")]) <= 0)  # stronger damping at larger n
        if corr:
            assert np.all(ten[n == 1] == 0) and np.all(imp[n == 1] == 1.0)  # rigid rotation kept
        # order 8: D_n / D_N = (n(n+1) / N(N+1))^4 without the correction
        if not corr:
            assert np.allclose(ten / ten[top][0], (n * (n + 1.0) / (N * (N + 1.0))) ** 4, rtol=1e-13)
    with pytest.raises(ValueError):
        oracle.spec_apply(N, oracle.SPEC_HDIFF_IMPLICIT, s, A, 7, TAU, DT)


GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "spec_ops_t21.npz")


def test_oracle_matches_golden(oracle):
    """The C oracle against the independent numpy restatement's fixture
    (tests/golden/make_golden.py, spec_numpy)."""
    g = np.load(GOLDEN)
    N, a, order, tau, dt = int(g["N"]), float(g["a"]), int(g["order"]), float(g["tau"]), float(g["dt"])
    for kind in range(4):
        for corr in (0, 1):
            want = g["out_%d_%d" % (kind, corr)]
            got = oracle.spec_apply(N, kind, g["spec"], a, order, tau, dt, corr)
            assert np.abs(got - want).max() <= 1e-14 * np.abs(want).max(), (kind, corr)


@pytest.mark.gpu
def test_spec_ops_match_golden(dccm, cuda):
    g = np.load(GOLDEN)
    N, a, order, tau, dt = int(g["N"]), float(g["a"]), int(g["order"]), float(g["tau"]), float(g["dt"])
    for kind in range(4):
        for corr in (0, 1):
            want = g["out_%d_%d" % (kind, corr)]
            got = dccm.spec_apply(N, dccm.spec_op(kind, a, order, tau, dt, corr), g["spec"])
            assert np.abs(got - want).max() <= 1e-14 * np.abs(want).max(), (kind, corr)


CASES = [(21, 7), (85, 128), (341, 5), (0, 3)]


@pytest.mark.gpu
@pytest.mark.parametrize("N,batch", CASES)
@pytest.mark.parametrize("kind", [0, 1, 2, 3])
def test_spec_ops_match_oracle(dccm, oracle, synth, cuda, N, batch, kind):
    if N < 2 and kind >= 2:
        pytest.skip("hyperdiffusion needs nmax >= 2")
    s = synth.spectra(N, batch, seed=N + kind)
    if N == 0:
        s[:] = 2.0 + 1.0j
    for corr in (False, True) if kind >= 2 else (False,):
        op = dccm.spec_op(kind, A, 8, TAU, DT, corr)
        got = dccm.spec_apply(N, op, s)
        want = oracle.spec_apply(N, kind, s, A, 8, TAU, DT, corr)
        scale = max(np.abs(want).max(), 1e-300)
        assert np.abs(got - want).max() <= 1e-14 * scale, (N, kind, corr)
    # in place on the device, stream-ordered
    torch = cuda
    d = torch.from_numpy(s.view(np.float64).copy()).cuda()
    op = dccm.spec_op(kind, A, 8, TAU, DT, True)
    dccm.spec_apply_dev(N, op, d, d, batch)
    torch.cuda.synchronize()
    want = oracle.spec_apply(N, kind, s, A, 8, TAU, DT, True)
    got = d.cpu().numpy().view(np.complex128)
    assert np.abs(got - want).max() <= 1e-14 * max(np.abs(want).max(), 1e-300)


@pytest.mark.gpu
def test_spec_ops_invalid(dccm, cuda):
    s = np.zeros((2, 253), np.complex128)
    for op in (dccm.spec_op(7, A), dccm.spec_op(0, -1.0), dccm.spec_op(3, A, 7, TAU, DT),
               dccm.spec_op(3, A, 8, 0.0, DT), dccm.spec_op(2, A, 0, TAU)):
        with pytest.raises(dccm.DccmError):
            dccm.spec_apply(21, op, s)
    with pytest.raises(dccm.DccmError):
        dccm.spec_apply(1, dccm.spec_op(3, A, 8, TAU, DT), np.zeros((1, 3), np.complex128))
    assert dccm.spec_apply(21, dccm.spec_op(0, A), np.zeros((0, 253), np.complex128)).shape == (0, 253)
