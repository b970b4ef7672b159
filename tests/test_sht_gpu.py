"""GPU parity of the spherical-harmonic transforms against the FP64 oracle,
through the C ABI.  Tolerances (relative L2 over the whole batch):
  FP64 plan   1e-13 (inverse grid, forward spectra), nodes 2e-16;
  mixed plan  1e-6  (BF16 x 3 Legendre on tcgen05, FP32 FFT);
  FP16 plan   1e-6  (FP16 hi + lo Legendre with per-m and per-field-level
              power-of-two scales, FP32 FFT)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, rel_l2

pytestmark = pytest.mark.gpu

TRUNC = [(21, 64, 32), (42, 128, 64), (63, 192, 96), (85, 256, 128)]


@pytest.mark.parametrize("N,I,J", TRUNC + [(341, 1024, 512)])
def test_gauss_and_pnm_match_oracle(dccm, oracle, N, I, J):
    plan = dccm.ShtPlan(N, I, J, dccm.SHT_FP64, 1)
    mu, w = plan.gauss()
    mo, wo = oracle.gauss_nodes(J)
    assert np.abs(mu - mo).max() <= 2e-16
    assert np.abs(w - wo).max() <= 1e-15
    assert abs(w.sum() - 2.0) <= 1e-13
    lon, lat, lw, yw = plan.axes()
    assert np.allclose(np.sin(lat), mu, atol=1e-15) and np.all(yw == w)
    assert np.allclose(lon, 2 * np.pi * np.arange(I) / I) and np.allclose(lw, 2 * np.pi / I)
    p = plan.pnm()
    po = oracle.pnm(N, J)[:, J // 2:]
    assert np.abs(p - po).max() <= 1e-11 * max(1.0, np.abs(po).max())


@pytest.mark.parametrize("N,I,J", TRUNC)
def test_fp64_transforms_match_oracle(dccm, oracle, synth, N, I, J):
    B = 6
    s = synth.spectra(N, B, seed=N)
    plan = dccm.ShtPlan(N, I, J, dccm.SHT_FP64, B)
    g = plan.inverse(s)
    go = oracle.sht_inverse(N, I, J, s)
    assert rel_l2(g, go) <= 1e-13
    s2 = plan.forward(go)
    so = oracle.sht_forward(N, I, J, go)
    assert rel_l2(s2, so) <= 1e-13
    assert rel_l2(plan.forward(g), s) <= 1e-13


MIXED = [1, 2]  # SHT_MIXED (BF16 x 3), SHT_MIXED_FP16


@pytest.mark.parametrize("prec", MIXED)
@pytest.mark.parametrize("N,I,J", TRUNC)
def test_mixed_transforms_match_oracle(dccm, oracle, synth, N, I, J, prec):
    B = 70  # two 128-column blocks of the batch, the second partial
    s = synth.spectra(N, B, seed=N + 1)
    plan = dccm.ShtPlan(N, I, J, prec, B)
    g = plan.inverse(s)
    go = oracle.sht_inverse(N, I, J, s)
    e_inv = rel_l2(g, go)
    s2 = plan.forward(go)
    so = oracle.sht_forward(N, I, J, go)
    e_fwd = rel_l2(s2, so)
    e_rt = rel_l2(plan.forward(g), s)
    assert plan.status() == (0, 0)
    assert e_inv <= 1e-6 and e_fwd <= 1e-6 and e_rt <= 1e-6, (e_inv, e_fwd, e_rt)
    # per field-level, not only in aggregate
    for b in range(0, B, 7):
        assert rel_l2(g[b], go[b]) <= 2e-6
        assert rel_l2(s2[b], so[b]) <= 2e-6


# Longer rows: I = 32 R with R = 12 (one warp per row pair, 12 samples a
# lane) and R = 16, 24, 32 (rows shared by 2, 3, 4 warps).  Six field-levels
# leave the last CTA of field-levels partial for every layout.  The
# tolerance grows with N (BF16 x 3 Legendre sums over up to N/2 terms,
# FP32 FFT of length I): 2e-6 over the batch, 4e-6 per field-level.
LONG = [(127, 384, 192), (170, 512, 256), (255, 768, 384), (341, 1024, 512)]


@pytest.mark.parametrize("prec", MIXED)
@pytest.mark.parametrize("N,I,J", LONG)
def test_mixed_long_rows_match_oracle(dccm, oracle, synth, N, I, J, prec):
    B = 6
    s = synth.spectra(N, B, seed=N + 3)
    plan = dccm.ShtPlan(N, I, J, prec, B)
    g = plan.inverse(s)
    go = oracle.sht_inverse(N, I, J, s)
    s2 = plan.forward(go)
    so = oracle.sht_forward(N, I, J, go)
    errs = (rel_l2(g, go), rel_l2(s2, so), rel_l2(plan.forward(g), s))
    assert plan.status() == (0, 0)
    assert max(errs) <= 2e-6, errs
    for b in range(B):
        assert rel_l2(g[b], go[b]) <= 4e-6
        assert rel_l2(s2[b], so[b]) <= 4e-6


@pytest.mark.parametrize("prec", [0, 1, 2])
def test_known_answers(dccm, oracle, prec):
    N, I, J = 21, 64, 32
    plan = dccm.ShtPlan(N, I, J, prec, 3)
    mu, w = plan.gauss()
    lon = 2 * np.pi * np.arange(I) / I
    s = np.zeros((3, (N + 1) * (N + 2) // 2), complex)
    s[0, 1] = 1.0          # Y_1^0 = sqrt(3) mu
    s[1, N + 1] = 1.0      # s_1^1 = 1: 2 sqrt(3/2) cos(lat) cos(lon)
    s[2, 2] = 1.0          # Y_2^0 = sqrt(5)/2 (3 mu^2 - 1)
    g = plan.inverse(s)
    tol = 1e-13 if prec == 0 else 1e-6
    assert np.abs(g[0] - np.sqrt(3) * mu[:, None]).max() <= tol * 2
    ref = 2 * np.sqrt(1.5) * np.sqrt(1 - mu ** 2)[:, None] * np.cos(lon)[None, :]
    assert np.abs(g[1] - ref).max() <= tol * 3
    assert np.abs(g[2] - (np.sqrt(5) / 2 * (3 * mu ** 2 - 1))[:, None]).max() <= tol * 3
    back = plan.forward(g)
    assert np.abs(back - s).max() <= tol * 3


@pytest.mark.parametrize("prec", [0, 1, 2])
def test_golden_fixture(dccm, prec):
    z = np.load(os.path.join(GOLDEN, "sht_t21.npz"))
    N, I, J = int(z["N"]), int(z["I"]), int(z["J"])
    plan = dccm.ShtPlan(N, I, J, prec, 3)
    tol = 1e-13 if prec == 0 else 1e-6
    assert rel_l2(plan.inverse(z["spec"]), z["grid"]) <= tol
    assert rel_l2(plan.forward(z["grid"]), z["fwd"]) <= tol


def test_device_entry_points(dccm, oracle, synth, cuda):
    torch = cuda
    N, I, J, B = 85, 256, 128, 128
    s = synth.spectra(N, B, seed=3)
    for prec, tol in ((0, 1e-13), (1, 1e-6)):
        plan = dccm.ShtPlan(N, I, J, prec, B)
        ds = torch.from_numpy(s.view(np.float64).copy()).cuda()
        dg = torch.empty((B, J, I), dtype=torch.float64, device="cuda")
        ds2 = torch.empty_like(ds)
        st = torch.cuda.current_stream()
        plan.inverse_dev(ds, dg, B, st)
        plan.forward_dev(dg, ds2, B, st)
        torch.cuda.synchronize()
        s2 = ds2.cpu().numpy().view(np.complex128)
        assert rel_l2(s2, s) <= tol
        assert plan.status() == (0, 0)


def test_batch_limits(dccm):
    plan = dccm.ShtPlan(21, 64, 32, 0, 2)
    with pytest.raises(dccm.DccmError) as e:
        plan.inverse(np.zeros((3, 253), complex))
    assert e.value.status == -2
    with pytest.raises(dccm.DccmError):
        dccm.ShtPlan(21, 40, 32, 0, 1)  # imax <= 2 nmax
    with pytest.raises(dccm.DccmError):
        dccm.ShtPlan(21, 70, 32, 0, 1)  # 70 = 2 * 5 * 7 is not 2^a 3^b


@pytest.mark.parametrize("prec", MIXED)
def test_mixed_field_magnitudes(dccm, oracle, synth, prec):
    """Field-levels of very different magnitude in one batch (a vorticity
    of 1e-5, a temperature of 300, a pressure of 1e5, and 1e-12): every
    field-level keeps its relative accuracy (the FP16 plan scales each
    field-level into FP16's range on its own)."""
    N, I, J, B = 85, 256, 128, 8
    s = synth.spectra(N, B, seed=11)
    mags = np.array([1e-5, 300.0, 1e5, 1e-12, 1.0, 3e-3, 7e2, 2e-8])
    s = s * mags[:, None]
    plan = dccm.ShtPlan(N, I, J, prec, B)
    g = plan.inverse(s)
    go = oracle.sht_inverse(N, I, J, s)
    s2 = plan.forward(go)
    so = oracle.sht_forward(N, I, J, go)
    assert plan.status() == (0, 0)
    for b in range(B):
        assert rel_l2(g[b], go[b]) <= 2e-6, (b, rel_l2(g[b], go[b]))
        assert rel_l2(s2[b], so[b]) <= 2e-6, (b, rel_l2(s2[b], so[b]))


@pytest.mark.parametrize("prec", [0, 1, 2])
def test_zero_and_single_field_level(dccm, oracle, synth, cuda, prec):
    """batch 0 is a no-op that leaves the output untouched; batch 1 uses one
    ragged column block (1 of 128 columns) of every tensor-core item."""
    torch = cuda
    N, I, J = 42, 128, 64
    plan = dccm.ShtPlan(N, I, J, prec, 4)
    s = synth.spectra(N, 1, seed=21)
    ds = torch.from_numpy(s.view(np.float64).copy()).cuda()
    dg = torch.full((1, J, I), 7.0, dtype=torch.float64, device="cuda")
    plan.inverse_dev(ds, dg, 0)
    torch.cuda.synchronize()
    assert bool((dg == 7.0).all())
    tol = 1e-13 if prec == 0 else 1e-6
    g = plan.inverse(s)
    go = oracle.sht_inverse(N, I, J, s)
    assert rel_l2(g, go) <= tol
    assert rel_l2(plan.forward(go), oracle.sht_forward(N, I, J, go)) <= tol
    assert plan.status() == (0, 0)


@pytest.mark.parametrize("rpw,bb", [(2, 4), (2, 8), (2, 16), (1, 4)])
@pytest.mark.parametrize("N,I,J", TRUNC + LONG)
def test_fft_launch_shapes_match_oracle(dccm, oracle, synth, N, I, J, rpw, bb):
    """Every FFT launch shape the autotuner can pick (warps per CTA, two
    row pairs a warp or a warp group in turn): the same results, with a
    batch that leaves the last CTA of field-levels partial (13 field-levels,
    CTAs of 1 to 32)."""
    B = 13
    s = synth.spectra(N, B, seed=N + 5)
    saved = {k: dccm.tune_get(k) for k in ("fft_rpw", "fft_bb")}
    try:
        dccm.tune_set("fft_rpw", rpw)
        dccm.tune_set("fft_bb", bb)
        plan = dccm.ShtPlan(N, I, J, 1, B)
        g = plan.inverse(s)
        go = oracle.sht_inverse(N, I, J, s)
        s2 = plan.forward(go)
        so = oracle.sht_forward(N, I, J, go)
        assert plan.status() == (0, 0)
        assert rel_l2(g, go) <= 2e-6 and rel_l2(s2, so) <= 2e-6
        for b in range(B):
            assert rel_l2(g[b], go[b]) <= 4e-6 and rel_l2(s2[b], so[b]) <= 4e-6, b
    finally:
        for k, v in saved.items():
            dccm.tune_set(k, v)
