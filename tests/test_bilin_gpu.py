"""GPU parity of the bilinear table generator and the surface exchange grid
against the oracle, through the C ABI: rows and weights bit-exact (the GPU
evaluates the reference's expressions in the same order), exchange-grid
latitudes and widths bit-exact; and the six gmapgen tables end to end."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

CASES = ["t21_to_t42", "t42_to_t21", "t21_to_reg", "axi_dst", "axi_src"]


def _case(z, name):
    g = z[name + "_grid"]
    o = np.cumsum([0] + list(g))
    ll = z[name + "_lon_lat"]
    return [ll[o[i]:o[i + 1]] for i in range(4)]


def _rows(t):
    iD, jD, iS, jS, w = t.rows()
    return np.stack([iD, jD, iS, jS], 1), w


@pytest.mark.parametrize("name", CASES)
def test_bilinear_golden(dccm, name):
    z = np.load(os.path.join(GOLDEN, "bilin_small.npz"))
    lonS, latS, lonR, latR = _case(z, name)
    idx, w = _rows(dccm.bilinear_generate(lonS, latS, lonR, latR))
    assert np.array_equal(idx, z[name + "_idx"])
    assert np.array_equal(w, z[name + "_w"])


@pytest.mark.parametrize("src,dst", [((256, 128), (360, 180)), ((1024, 512), (1440, 720)),
                                     ((360, 180), (256, 128))])
def test_bilinear_large_matches_oracle(dccm, oracle, synth, src, dst):
    S = synth.gaussian_axes(*src) if src[0] in (256, 1024) else synth.regular_axes(*src)
    R = synth.regular_axes(*dst) if dst[0] in (360, 1440) else synth.gaussian_axes(*dst)
    o = oracle.bilin_gen(S[0], S[1], R[0], R[1])
    idx, w = _rows(dccm.bilinear_generate(S[0], S[1], R[0], R[1]))
    assert np.array_equal(idx, np.stack(o[:4], 1))
    assert np.array_equal(w, o[4])


def test_bilinear_mask_and_apply(dccm, oracle, synth):
    """Masked destination rows are dropped; the table applies through the
    same CSR path as Jones-99 tables, bit-exact against the oracle."""
    S = synth.gaussian_axes(128, 64)
    R = synth.regular_axes(180, 90)
    mask = synth.land_mask(180, 90, 0.3, seed=1)
    full = dccm.bilinear_generate(S[0], S[1], R[0], R[1]).rows()
    t = dccm.bilinear_generate(S[0], S[1], R[0], R[1], dst_mask=mask)
    iD, jD, iS, jS, w = t.rows()
    keep = mask[(full[0] - 1) + 180 * (full[1] - 1)] == 1
    assert np.array_equal(iD, full[0][keep]) and np.array_equal(w, full[4][keep])
    send, recv, coef = t.index(128, 180)
    plan = dccm.RemapPlan(128 * 64, 180 * 90, send, recv, coef)
    rng = np.random.Generator(np.random.PCG64(0))
    src = np.asfortranarray(rng.normal(size=(128 * 64, 3)))
    got = np.zeros((180 * 90, 3), order="F")
    plan.interpolate_data(src, got, 3)
    ref = oracle.remap_apply(send, recv, coef, src, 180 * 90)
    assert np.array_equal(got, ref)


def test_exchange_grid_and_gmapgen(dccm, oracle, synth):
    A = synth.gaussian_axes(64, 32)
    O = synth.regular_axes(128, 64)
    lat, w = dccm.exchange_grid(A[1], A[3], O[1], O[3])
    lo, wo = oracle.exchange_grid_lat(A[1], A[3], O[1], O[3])
    assert np.array_equal(lat, lo) and np.array_equal(w, wo)
    same = dccm.exchange_grid(A[1], A[3], A[1], A[3])
    assert np.array_equal(same[0], A[1]) and np.array_equal(same[1], A[3])
    for conservative in (True, False):
        S, tabs = dccm.gmapgen(A, O, conservative=conservative)
        assert set(tabs) == {"AO", "OA", "AS", "SA", "OS", "SO"}
        assert np.array_equal(S[1], lat)
        for tag, t in tabs.items():
            assert len(t.rows()[4]) > 0, tag
    # conservative AS: the exchange grid refines A, so every S cell has rows
    S, tabs = dccm.gmapgen(A, O, conservative=True, weight_mode=dccm.J99_CONSERVE)
    iD, jD, iS, jS, wt = tabs["AS"].rows()
    sums = np.zeros(len(S[0]) * len(S[1]))
    np.add.at(sums, (iD - 1) + len(S[0]) * (jD - 1), wt)
    assert np.allclose(sums, 1.0, atol=1e-12)
