"""CPU tests: the oracle against the golden fixtures (an independent numpy
restatement, tests/golden/make_golden.py) and against analytic known answers.
No GPU is used."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, rel_l2


def _flux_case():
    z = np.load(os.path.join(GOLDEN, "flux_small.npz"))
    IA, JA, IS, IE, JS, JE = (int(z[k]) for k in ("IA", "JA", "IS", "IE", "JS", "JE"))
    ins = {k[3:]: np.asfortranarray(z[k]) for k in z.files if k.startswith("in_")}
    outs = {k[4:]: z[k] for k in z.files if k.startswith("out_")}
    return (IA, JA, IS, IE, JS, JE), ins, outs


def _flux_outputs(IA, JA):
    out = {n: np.full((IA, JA, 3), -777.0, order="F") for n in (
        "WindStressX", "WindStressY", "SenHFlx", "QVapMFlx", "LatHFlx", "SfcVelTransCoef", "SfcTempTransCoef",
        "SfcQVapTransCoef", "SUwRFlx", "LUwRFlx", "SfcHFlx_ns", "SfcHFlx_sr", "DSfcHFlxDTs")}
    out["DelVarImplCPL"] = np.full((IA, JA, 4), -777.0, order="F")
    return out


def test_flux_oracle_matches_golden(oracle):
    (IA, JA, IS, IE, JS, JE), ins, gold = _flux_case()
    arrs = dict(ins)
    arrs["SfcTemp"] = ins["SfcTemp"].copy(order="F")
    arrs["SfcAlbedo"] = ins["SfcAlbedo"].copy(order="F")
    arrs.update(_flux_outputs(IA, JA))
    oracle.sfc_bulk_flux(arrs, IA, JA, IS, IE, JS, JE)
    it = (slice(IS - 1, IE), slice(JS - 1, JE))
    for name in ("WindStressX", "WindStressY", "SenHFlx", "QVapMFlx", "LatHFlx", "SfcVelTransCoef",
                 "SfcTempTransCoef", "SfcQVapTransCoef", "SUwRFlx", "LUwRFlx", "DelVarImplCPL"):
        got = arrs[name][it]
        assert rel_l2(got, gold[name]) <= 1e-13, name
        assert np.allclose(got, gold[name], rtol=1e-12, atol=1e-300), name
    for name in ("SfcHFlx_ns", "SfcHFlx_sr", "DSfcHFlxDTs"):
        assert rel_l2(arrs[name][it][..., :2], gold[name]) <= 1e-13, name
        # slot 3 untouched (the reference's final loop covers n = 1..2)
        assert np.all(arrs[name][..., 2] == -777.0), name
    assert rel_l2(arrs["SfcTemp"][it][..., 2], gold["SfcTemp3"]) <= 1e-14
    assert rel_l2(arrs["SfcAlbedo"][it][..., 2], gold["SfcAlbedo3"]) <= 1e-14
    # halo cells untouched
    for name in ("WindStressX", "DelVarImplCPL"):
        a = arrs[name]
        assert np.all(a[0] == -777.0) and np.all(a[-1] == -777.0) and np.all(a[:, 0] == -777.0)


def test_flux_known_answers(oracle):
    """Single columns: stable (Ri>0) and unstable branches, absent ice
    (outputs of slot 2 are 0) and the velocity floor."""
    (IA, JA, IS, IE, JS, JE), ins, gold = _flux_case()
    arrs = dict(ins)
    arrs["SfcTemp"] = ins["SfcTemp"].copy(order="F")
    arrs["SfcAlbedo"] = ins["SfcAlbedo"].copy(order="F")
    arrs.update(_flux_outputs(IA, JA))
    oracle.sfc_bulk_flux(arrs, IA, JA, IS, IE, JS, JE)
    ice = ins["SIceCon"]
    no_ice = (ice[1:-1, 1:-1] <= 1e-12)
    assert no_ice.any()
    for name in ("WindStressX", "SenHFlx", "LatHFlx", "LUwRFlx", "SUwRFlx"):
        assert np.all(arrs[name][1:-1, 1:-1, 1][no_ice] == 0.0), name
    for name in ("SfcHFlx_ns", "SfcHFlx_sr", "DSfcHFlxDTs"):
        assert np.all(arrs[name][1:-1, 1:-1, 1][no_ice] == 0.0), name
    # Hand evaluation of one stable column over sea (column index chosen
    # with warm air: Ri > 0) of the reference's neutral/Louis formulas.
    i, j = 3, 2
    Ps, Ta, q1 = ins["SfcPress"][i, j], ins["SfcAirTemp"][i, j], ins["QVap1"][i, j]
    U, V, Ts = ins["WindU"][i, j], ins["WindV"][i, j], ins["SfcTemp"][i, j, 0]
    sig1 = ins["a_Sig1Info"][0]
    Rd, Rw, cp, g = 8.3144621 / 1.8e-2, 8.3144621 / 1.8e-2, 1616.0, 9.8
    qs = 611.0 / Ps * np.exp(2425300.0 / Rw * (1 / 273.0 - 1 / Ts))
    ex1, exs = (Ps * sig1 / 1e5) ** (Rd / cp), (Ps / 1e5) ** (Rd / cp)
    H = Rd / g * Ta * (1 - sig1)
    vabs = np.hypot(U, V)
    cmn = (0.4 / np.log((H + 1e-4) / 1e-4)) ** 2
    Ri = g / (Ts / exs) * (Ta / ex1 - Ts / exs) / max(vabs, 0.01) ** 2 * H
    assert Ri > 0
    cm = cmn / (1 + 10 * Ri / np.sqrt(1 + 5 * Ri))
    cvel = cm * Ps / (Rd * Ts) * min(max(vabs, 0.01), 1000.0)
    assert np.isclose(arrs["SfcVelTransCoef"][i, j, 0], cvel, rtol=1e-13)
    # calm column: the Richardson-number floor VelMinForRi = 0.01 applies
    assert ins["WindU"][4, 2] == 0.0 and ins["WindV"][4, 2] == 0.0
    assert arrs["SfcVelTransCoef"][4, 2, 0] > 0


def test_j99_oracle_matches_golden(oracle):
    z = np.load(os.path.join(GOLDEN, "j99_small.npz"))
    names = sorted({k.rsplit("_", 1)[0] for k in z.files})
    assert len(names) == 5
    for name in names:
        nxs, nys, nxd, nyd, order = (int(x) for x in z[name + "_shape"])
        g = z[name + "_grid"]
        o = 0
        lonS, latS, wS = g[o:o + nxs], g[o + nxs:o + nxs + nys], g[o + nxs + nys:o + nxs + 2 * nys]
        o = nxs + 2 * nys
        lonD, latD, wD = g[o:o + nxd], g[o + nxd:o + nxd + nyd], g[o + nxd + nyd:o + nxd + 2 * nyd]
        iD, jD, iS, jS, w = oracle.j99_gen(lonS, latS, lonD, latD, wS, wD, order, 0)
        idx = z[name + "_idx"]
        assert len(w) == len(z[name + "_w"]), name
        assert np.array_equal(np.stack([iD, jD, iS, jS], 1), idx), name
        assert np.array_equal(w, z[name + "_w"]), name  # same formula, same libm: bit-exact


def test_j99_reference_defects_reproduced(oracle, synth):
    """D1: refining in longitude gives row sums of 2; coarsening writes
    source indices <= 0 for the wrap-around cell."""
    lonS, latS, _, wS = synth.gaussian_axes(64, 32)
    lonD, latD, _, wD = synth.gaussian_axes(128, 64)
    iD, jD, iS, jS, w = oracle.j99_gen(lonS, latS, lonD, latD, wS, wD, 1, 0)
    rs = np.zeros(128 * 64)
    np.add.at(rs, (iD - 1) + 128 * (jD - 1), w)
    assert np.isclose(rs.max(), 2.0) and np.isclose(rs.min(), 1.0)
    iD, jD, iS, jS, w = oracle.j99_gen(lonD, latD, lonS, latS, wD, wS, 1, 0)
    assert (iS <= 0).sum() > 0 and np.all(iD[iS <= 0] == 1)
    # conservative mode: row sums 1 in both directions
    for a, b in (((lonS, latS, wS), (lonD, latD, wD)), ((lonD, latD, wD), (lonS, latS, wS))):
        iD, jD, iS, jS, w = oracle.j99_gen(a[0], a[1], b[0], b[1], a[2], b[2], 1, 1)
        nx = len(b[0])
        rs = np.zeros(nx * len(b[1]))
        np.add.at(rs, (iD - 1) + nx * (jD - 1), w)
        assert np.abs(rs - 1).max() < 1e-13
        assert iS.min() >= 1


def test_remap_apply_oracle_identity_fixture(oracle, synth):
    """The exchange-debug pattern i + 100 j + 1e4 code (common/field_def.f90:586)
    through the identity T42 table comes back bit-exact."""
    lon, lat, _, w = synth.gaussian_axes(128, 64)
    iD, jD, iS, jS, cw = oracle.j99_gen(lon, lat, lon, lat, w, w, 1, 0)
    assert len(cw) == 128 * 64 and np.all(cw == 1.0)
    send, recv = oracle.table_to_index(iD, jD, iS, jS, 128, 128)
    ii, jj = np.meshgrid(np.arange(1, 129), np.arange(1, 65), indexing="ij")
    fields = np.stack([(ii + 100 * jj + 1e4 * code).ravel(order="F") for code in range(1, 7)], 1)
    out = oracle.remap_apply(send, recv, cw, np.asfortranarray(fields), 128 * 64)
    assert np.array_equal(out, fields)


def test_gauss_nodes_vs_numpy(oracle):
    for J in (32, 64, 96, 128, 512):
        mu, w = oracle.gauss_nodes(J)
        x, wx = np.polynomial.legendre.leggauss(J)
        assert np.abs(mu - x).max() <= 2e-16
        assert np.abs(w - wx).max() <= 1e-14
        assert abs(w.sum() - 2.0) <= 1e-14  # the reference's own check (gmapgen_main.f90:403)
        assert np.array_equal(mu, -mu[::-1])


def test_sht_oracle_matches_golden(oracle):
    z = np.load(os.path.join(GOLDEN, "sht_t21.npz"))
    N, I, J = int(z["N"]), int(z["I"]), int(z["J"])
    p = oracle.pnm(N, J)
    assert np.abs(p - z["pbar"]).max() <= 1e-13
    g = oracle.sht_inverse(N, I, J, z["spec"])
    assert rel_l2(g, z["grid"]) <= 1e-14
    s = oracle.sht_forward(N, I, J, z["grid"])
    assert rel_l2(s, z["fwd"]) <= 1e-14
    assert rel_l2(s, z["spec"]) <= 1e-13


@pytest.mark.parametrize("N,I,J", [(21, 64, 32), (42, 128, 64), (63, 192, 96), (85, 256, 128)])
def test_sht_oracle_round_trip_and_analytic(oracle, synth, N, I, J):
    s = synth.spectra(N, 2, seed=N)
    g = oracle.sht_inverse(N, I, J, s)
    s2 = oracle.sht_forward(N, I, J, g)
    assert rel_l2(s2, s) <= 1e-13
    mu, w = oracle.gauss_nodes(J)
    lon = 2 * np.pi * np.arange(I) / I
    one = np.zeros((1, synth.ncoef(N)), complex)
    one[0, 1] = 1.0  # Y_1^0 = sqrt(3) mu
    assert np.abs(oracle.sht_inverse(N, I, J, one)[0] - np.sqrt(3) * mu[:, None]).max() <= 1e-14
    one[:] = 0
    one[0, N + 1] = 1.0  # s_1^1 = 1 -> 2 sqrt(3/2) cos(lat) cos(lon)
    ref = 2 * np.sqrt(1.5) * np.sqrt(1 - mu ** 2)[:, None] * np.cos(lon)[None, :]
    assert np.abs(oracle.sht_inverse(N, I, J, one)[0] - ref).max() <= 1e-13
    one[:] = 0
    one[0, 2] = 1.0  # Y_2^0 = sqrt(5)/2 (3 mu^2 - 1)
    ref = np.sqrt(5) / 2 * (3 * mu ** 2 - 1)
    assert np.abs(oracle.sht_inverse(N, I, J, one)[0] - ref[:, None]).max() <= 1e-13
    # orthonormality: (1/2) sum_j w_j Pbar_n^m Pbar_n'^m = delta
    p = oracle.pnm(N, J)
    for m in (0, 1, N // 2, N):
        rows = [sum(N + 1 - k for k in range(m)) + (n - m) for n in range(m, N + 1)]
        G = 0.5 * (p[rows] * w) @ p[rows].T
        assert np.abs(G - np.eye(len(rows))).max() <= 1e-12


def test_area_integral_compensated(oracle):
    rng = np.random.default_rng(5)
    f = rng.standard_normal(100000) * 1e8
    f = np.concatenate([f, -f, [1.0]])
    a = np.ones_like(f)
    assert oracle.area_integral(f, a) == 1.0


# ------------------------------------------------------ implicit coupling
def _same(a, g):
    """Bit-identical finite values; same infinities (with sign) and NaN."""
    fin = np.isfinite(g)
    return (np.array_equal(np.isfinite(a), fin) and np.array_equal(np.isnan(a), np.isnan(g))
            and np.array_equal(np.signbit(a[~fin]), np.signbit(g[~fin])) and np.array_equal(a[fin], g[fin]))


def test_implcpl_forward_matches_golden(oracle):
    z = np.load(os.path.join(GOLDEN, "implcpl_small.npz"))
    d = {k[3:]: z[k] for k in z.files if k.startswith("in_")}
    o = oracle.implcpl_forward(d, int(z["ih2o"]), z["consts"])
    for k, v in o.items():
        assert _same(v, z["out_" + k]), k
    # the reference's level-1 division by its zero sub-diagonal (only there)
    assert not np.isfinite(o["DUDt"][0]).any() and np.isfinite(o["DUDt"][1:]).all()
    assert np.isfinite(o["ImplCplCoef1"]).all() and np.isfinite(o["ImplCplCoef2"]).all()


def test_implcpl_sweeps_solve_the_column_systems(oracle, synth):
    """Forward elimination, a surface value at level 1 (as the coupler puts
    DelVarImplCPL there) and back substitution solve rows 2..kmax of the
    original momentum system: A x = -(flux divergence), x = 2 dt dU/dt."""
    ncol = 40
    d = synth.column_profiles(ncol, 20, ncmax=2, seed=9)
    G, Cp, R, DT = synth.IMPLCPL_CONSTS
    o = oracle.implcpl_forward(d, 1, synth.IMPLCPL_CONSTS)
    rng = np.random.Generator(np.random.PCG64(3))
    t = {k: o[k].copy() for k in ("DUDt", "DVDt", "DTempDt", "DQMixDt")}
    for k in ("DUDt", "DVDt", "DTempDt"):
        t[k][0] = rng.normal(0, 1e-3, ncol)
    t["DQMixDt"][:, 0] = rng.normal(0, 1e-7, (2, ncol))
    b = oracle.implcpl_backward(o, t, DT)
    assert all(np.isfinite(v).all() for v in b.values())
    K = d["Press"].shape[0] - 1
    VTC = np.zeros((K + 1, ncol))
    for k in range(1, K):
        VTC[k] = d["VelDiffCoef"][k] * (d["Press"][k] / (R * d["VirTemp"][k]) / (d["Height"][k] - d["Height"][k - 1]))
    rhs = -(d["MomFluxX"][1:] - d["MomFluxX"][:-1])
    x = b["DUDt"] * (2.0 * DT)
    for k in range(2, K + 1):
        mass = -((d["Press"][k] - d["Press"][k - 1]) / G / (2.0 * DT))
        m0 = mass + VTC[k - 1] + (VTC[k] if k < K else 0.0)
        lhs = -VTC[k - 1] * x[k - 2] + m0 * x[k - 1] + (-VTC[k] * x[k] if k < K else 0.0)
        assert np.allclose(lhs, rhs[k - 1], rtol=1e-9, atol=1e-12 * np.abs(rhs).max()), k


# -------------------------------------------- bilinear table, exchange grid
BILIN_CASES = ["t21_to_t42", "t42_to_t21", "t21_to_reg", "axi_dst", "axi_src"]


def bilin_case(z, name):
    g = z[name + "_grid"]
    o = np.cumsum([0] + list(g))
    ll = z[name + "_lon_lat"]
    return [ll[o[i]:o[i + 1]] for i in range(4)]


@pytest.mark.parametrize("name", BILIN_CASES)
def test_bilinear_matches_golden(oracle, name):
    z = np.load(os.path.join(GOLDEN, "bilin_small.npz"))
    lonS, latS, lonR, latR = bilin_case(z, name)
    r = oracle.bilin_gen(lonS, latS, lonR, latR)
    assert np.array_equal(np.stack(r[:4], 1), z[name + "_idx"])
    assert np.array_equal(r[4], z[name + "_w"])
    # every destination cell's weights sum to 1 (interpolation, extrapolation)
    nxr = len(lonR)
    s = np.zeros(nxr * len(latR))
    np.add.at(s, (r[0] - 1) + nxr * (r[1] - 1), r[4])
    assert np.allclose(s, 1.0, atol=1e-13)


def test_exchange_grid_matches_golden(oracle):
    z = np.load(os.path.join(GOLDEN, "bilin_small.npz"))
    mu, wA = np.polynomial.legendre.leggauss(32)
    e = np.linspace(-np.pi / 2, np.pi / 2, 65)
    lat, w = oracle.exchange_grid_lat(np.arcsin(mu), wA, 0.5 * (e[1:] + e[:-1]), np.sin(e[1:]) - np.sin(e[:-1]))
    assert np.array_equal(lat, z["xgrid_lat"]) and np.array_equal(w, z["xgrid_w"])
    assert abs(w.sum() - 2.0) < 1e-13 and np.all(np.diff(lat) > 0)
