"""Generates the golden fixtures in this folder.

The reference ships no golden vectors and cannot be compiled here (Fortran 90,
no Fortran compiler or jcup/gtool5/SPML libraries), so these fixtures come
from a second, independent restatement of the reference written in numpy /
plain Python, kept deliberately different in structure from the C oracle:

* bulk flux: array-at-a-time numpy over the whole grid, one loop nest per
  reference loop (sfc/DSFCM_Util_SfcBulkFlux_mod.f90:194-415, BulkCoefL82
  :443-572), serial meaning of the shared sea-ice flag (:384-393), slot-3
  latent heat as the fraction-weighted merge (the reference reads index 3 of
  an extent-2 array at :379);
* Jones-99 table: the Fortran loops transcribed line by line in Python,
  including the values search_OverwrapRange leaves unassigned
  (common/grid_mapping_util_jones99.f90:156-442);
* spherical harmonics: Legendre functions from scipy.special.lpmv (not the
  recurrence the oracle uses), Gaussian nodes from numpy.polynomial, and
  full-latitude sums without the equatorial fold; FFTs from numpy.fft;
* implicit surface coupling: whole levels of all columns at a time
  (atm/dcpam_sfc_implicit_coupling_mod.f90:72-405), the oracle loops per
  column;
* bilinear table and exchange grid: the Fortran loops transcribed in
  Python (common/grid_mapping_util.f90:32-182,
  tool/gmapgen/gmapgen_main.f90:336-405), Python's sort for the edges;
* spectral operators (Laplacian, inverse Laplacian, hyperdiffusion; the
  reference's code is external, so from the mathematics): factors as
  numpy powers of n(n+1) over a^order, the oracle multiplies per level.

Run from the repository root:  python tests/golden/make_golden.py
"""
import math
import os

import numpy as np
from scipy.special import lpmv

OUT = os.path.dirname(os.path.abspath(__file__))


# --------------------------------------------------------------- bulk flux
def flux_numpy(d, IA, JA, IS, IE, JS, JE):
    FKarm, GasRUniv, StB, Grav = 0.4, 8.3144621, 5.670373e-8, 9.8
    MolWtDry = MolWtWet = 1.8e-2
    CpDry, LatentHeat, LatentHeatFusion, RefPress, Es0 = 1616.0, 2425300.0, 334000.0, 1e5, 611.0
    RoughLength, RoughLenHeatFactor = 1e-4, 1.0
    GasRDry, GasRWet, EpsV = GasRUniv / MolWtDry, GasRUniv / MolWtWet, MolWtWet / MolWtDry
    vmin, vmax, cmin, cmax = 0.01, 1000.0, 0.0, 1.0
    s = (slice(IS - 1, IE), slice(JS - 1, JE))
    g = lambda k: d[k][s]
    g3 = lambda k, n: d[k][s + (n,)]
    aL = [LatentHeat, LatentHeat + LatentHeatFusion]
    Ps, Ta, q1, U, V, zs = g("SfcPress"), g("SfcAirTemp"), g("QVap1"), g("WindU"), g("WindV"), g("SfcHeight")
    sig1 = d["a_Sig1Info"][0]
    Frac = [1.0 - g("SIceCon"), g("SIceCon")]
    z0m = np.full(Ps.shape, RoughLength)
    z0h = RoughLenHeatFactor * z0m
    QSat, SVT = [], []
    for n in range(2):
        Ts = g3("SfcTemp", n)
        QSat.append(EpsV * Es0 / Ps * np.exp(aL[n] / GasRWet * (1.0 / 273.0 - 1.0 / Ts)))
        SVT.append(Ts * (1.0 + (((1.0 / EpsV) - 1.0) * QSat[n])))
    VT = Ta * (1.0 + (((1.0 / EpsV) - 1.0) * q1))
    Exner = (Ps * sig1 / RefPress) ** (GasRDry / CpDry)
    SExner = (Ps / RefPress) ** (GasRDry / CpDry)
    Vabs = np.sqrt(U ** 2 + V ** 2)
    H = zs + GasRDry / Grav * VT * (1.0 - sig1)
    out = {k: np.zeros(Ps.shape + (3,)) for k in ("WSX", "WSY", "Sen", "QV", "Lat", "CV", "CT", "CQ", "SUw", "LUw")}
    Ts3 = np.zeros(Ps.shape)
    Alb3 = np.zeros(Ps.shape)
    flags = []
    for n in range(2):
        tmp = FKarm / np.log((H - zs + z0m) / z0m)
        cmn = tmp ** 2
        chn = tmp * (FKarm / np.log((H - zs + z0h) / z0h))
        Ri = Grav / (SVT[n] / SExner) * (VT / Exner - SVT[n] / SExner) / np.maximum(Vabs, vmin) ** 2 * (H - zs)
        flag = np.ones(Ps.shape, bool) if n == 0 else Frac[n] > 1e-12
        flags.append(flag)
        with np.errstate(invalid="ignore"):
            st_m = cmn / (1.0 + 10.0 * Ri / np.sqrt(1.0 + 5.0 * Ri))
            st_h = chn / (1.0 + 15.0 * Ri * np.sqrt(1.0 + 5.0 * Ri))
            un_m = cmn * (1.0 - 10.0 * Ri / (1.0 + 75.0 * cmn * np.sqrt(-(H - zs + z0m) / z0m * Ri)))
            un_h = chn * (1.0 - 15.0 * Ri / (1.0 + 75.0 * chn * np.sqrt(-(H - zs + z0h) / z0h * Ri)))
        cm = np.where(flag, np.where(Ri > 0.0, st_m, un_m), 0.0)
        ch = np.where(flag, np.where(Ri > 0.0, st_h, un_h), 0.0)
        cm = np.maximum(np.minimum(cm, cmax), cmin)
        cq = np.maximum(np.minimum(ch, cmax), cmin)
        ch = np.maximum(np.minimum(ch, cmax), cmin)
        CV = cm * Ps / (GasRDry * SVT[n]) * np.minimum(np.maximum(Vabs, vmin), vmax)
        CT = ch * Ps / (GasRDry * SVT[n]) * np.minimum(np.maximum(Vabs, vmin), vmax)
        CQ = cq * Ps / (GasRDry * SVT[n]) * np.minimum(np.maximum(Vabs, vmin), vmax)
        out["CV"][..., n], out["CT"][..., n], out["CQ"][..., n] = CV, CT, CQ
        Ts = g3("SfcTemp", n)
        alb = g3("SfcAlbedo", n)
        wsx = np.where(flag, -CV * U, 0.0)
        wsy = np.where(flag, -CV * V, 0.0)
        sen = np.where(flag, -CpDry * SExner * CT * (Ta / Exner - Ts / SExner), 0.0)
        qv = np.where(flag, -1.0 * CQ * (q1 - QSat[n]), 0.0)
        lat = np.where(flag, aL[n] * qv, 0.0)
        luw = np.where(flag, StB * (Ts * Ts) * (Ts * Ts), 0.0)
        suw = np.where(flag, alb * g("SDwRFlx"), 0.0)
        for k, x in (("WSX", wsx), ("WSY", wsy), ("Sen", sen), ("QV", qv), ("Lat", lat), ("LUw", luw), ("SUw", suw)):
            out[k][..., n] = x
            out[k][..., 2] = np.where(flag, out[k][..., 2] + Frac[n] * x, out[k][..., 2])
        for k, x in (("CV", CV), ("CT", CT), ("CQ", CQ)):
            out[k][..., 2] = np.where(flag, out[k][..., 2] + Frac[n] * x, out[k][..., 2])
        Ts3 = np.where(flag, Ts3 + Frac[n] * (Ts * Ts) * (Ts * Ts), Ts3)
        Alb3 = np.where(flag, Alb3 + Frac[n] * alb, Alb3)
    c1 = [d["ImplCplCoef1"][s + (k,)] for k in range(4)]
    c2 = [d["ImplCplCoef2"][s + (k,)] for k in range(4)]
    DF = -CpDry * SExner * out["CT"][..., 2] / Exner
    gam = [1.0 / (c1[0] + out["CV"][..., 2]), 1.0 / (c1[1] + out["CV"][..., 2]),
           1.0 / (c1[2] - DF), 1.0 / (c1[3] + 1.0 * out["CQ"][..., 2])]
    f = [gam[0] * (out["WSX"][..., 2] + c2[0]), gam[1] * (out["WSY"][..., 2] + c2[1]),
         gam[2] * (out["Sen"][..., 2] + c2[2]), gam[3] * (out["QV"][..., 2] + c2[3])]
    for n in range(3):
        out["WSX"][..., n] = out["WSX"][..., n] - out["CV"][..., n] * f[0]
        out["WSY"][..., n] = out["WSY"][..., n] - out["CV"][..., n] * f[1]
        out["Sen"][..., n] = out["Sen"][..., n] - CpDry * SExner / Exner * out["CT"][..., n] * f[2]
        out["QV"][..., n] = out["QV"][..., n] - 1.0 * out["CQ"][..., n] * f[3]
        if n < 2:
            out["Lat"][..., n] = aL[n] * out["QV"][..., n]
    lat3 = np.zeros(Ps.shape)
    for n in range(2):
        lat3 = np.where(flags[n], lat3 + Frac[n] * out["Lat"][..., n], lat3)
    out["Lat"][..., 2] = lat3
    fns, fsr, dfdt = (np.zeros(Ps.shape + (2,)) for _ in range(3))
    for n in range(2):
        Ts = g3("SfcTemp", n)
        fl = flags[n]
        fns[..., n] = np.where(fl, +out["LUw"][..., n] - g("LDwRFlx") + out["Lat"][..., n] + out["Sen"][..., n], 0.0)
        fsr[..., n] = np.where(fl, out["SUw"][..., n] - g("SDwRFlx"), 0.0)
        dfdt[..., n] = np.where(fl, +4.0 * StB * (Ts * Ts * Ts) + CpDry * out["CT"][..., n]
                                + aL[n] * 1.0 * out["CQ"][..., n] * (aL[n] * QSat[n] / (GasRWet * (Ts * Ts))), 0.0)
    names = {"WSX": "WindStressX", "WSY": "WindStressY", "Sen": "SenHFlx", "QV": "QVapMFlx", "Lat": "LatHFlx",
             "CV": "SfcVelTransCoef", "CT": "SfcTempTransCoef", "CQ": "SfcQVapTransCoef", "SUw": "SUwRFlx",
             "LUw": "LUwRFlx"}
    res = {names[k]: v for k, v in out.items()}
    res["DelVarImplCPL"] = np.stack(f, axis=-1)
    res["SfcHFlx_ns"], res["SfcHFlx_sr"], res["DSfcHFlxDTs"] = fns, fsr, dfdt
    res["SfcTemp3"], res["SfcAlbedo3"] = Ts3, Alb3
    return res


def make_flux():
    import importlib
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(OUT)))
    synth = importlib.import_module("dennou-ccm_gb300.synth")
    nx, ny = 12, 8
    lat = np.deg2rad(np.linspace(-80, 80, ny))
    rng = np.random.Generator(np.random.PCG64(7))
    ice = np.where(rng.uniform(size=(nx, ny)) < 0.5, 0.0, rng.uniform(0, 1, (nx, ny)))
    ice[0, :] = 1e-13  # below the 1e-12 ice threshold
    ice[1, :] = 1.0
    d, (IA, JA, IS, IE, JS, JE) = synth.surface_state(lat, nx, seed=3, sea_ice=ice, halo_fill=0.0)
    # stable and unstable columns: warm / cold air over the sea surface
    d["SfcAirTemp"][1:-1, 1:5] += 6.0
    d["WindU"][1:-1, 2] = 0.0
    d["WindV"][1:-1, 2] = 0.0  # calm columns: velocity floors
    d["ImplCplCoef2"][1:-1, 1:-1, :] = rng.normal(0, 0.01, (nx, ny, 4))
    res = flux_numpy(d, IA, JA, IS, IE, JS, JE)
    ins = {k: v for k, v in d.items()}
    np.savez_compressed(os.path.join(OUT, "flux_small.npz"), IA=IA, JA=JA, IS=IS, IE=IE, JS=JS, JE=JE,
                        **{"in_" + k: v for k, v in ins.items()}, **{"out_" + k: v for k, v in res.items()})


# ------------------------------------------------------------- Jones-99
def j99_python(x_LonS, y_LatS, x_LonD, y_LatD, wS, wD, order):
    PI = math.acos(-1.0)

    def halo(lon, lat, latwt):
        nx, ny = len(lon), len(lat)
        IA, IS, IE, JA, JS, JE = nx + 2, 2, nx + 1, ny + 2, 2, ny + 1
        x = [0.0] * (IA + 2)
        y = [0.0] * (JA + 2)
        u = [0.0] * (IA + 2)
        v = [0.0] * (JA + 2)
        for i in range(IS, IE + 1):
            x[i] = float(lon[i - IS])
        for j in range(JS, JE + 1):
            y[j] = float(lat[j - JS])
        x[IS - 1] = x[IE] - 2.0 * PI
        x[IE + 1] = x[IS] + 2.0 * PI
        for i in range(IS - 1, IE + 1):
            u[i] = 0.5 * (x[i] + x[i + 1])
        v[JS - 1] = -PI / 2.0
        for j in range(JS, JE):
            v[j] = math.asin(float(latwt[j - JS]) + math.sin(v[j - 1]))
        v[JE] = PI / 2.0
        return x, y, u, v, IS, IE, JS, JE

    xS, yS, uS, vS, ISS, IES, JSS, JES = halo(x_LonS, y_LatS, wS)
    xD, yD, uD, vD, ISD, IED, JSD, JED = halo(x_LonD, y_LatD, wD)
    NXD, NXS = IED - ISD + 1, IES - ISS + 1
    rows = []
    X = [None, None]
    Y = [None, None]
    for jD in range(JSD, JED + 1):
        for iD in range(ISD, IED + 1):
            DX1, DX2, DY1, DY2 = uD[iD - 1], uD[iD], vD[jD - 1], vD[jD]
            X[0] = -1
            Y[1] = -1
            if NXS == 1 and NXD != 1:
                X = [ISS, ISS]
            elif NXS != 1 and NXD == 1:
                X = [ISS, IES]
            else:
                for i in range(ISS, IES + 1):
                    if uS[i - 1] <= DX1 <= uS[i]:
                        X[0] = i
                    if uS[i - 1] <= DX2 <= uS[i]:
                        X[1] = i
                        break
            for j in range(JSS, JES + 1):
                if vS[j - 1] <= DY1 <= vS[j]:
                    Y[0] = j
                if vS[j - 1] <= DY2 <= vS[j]:
                    Y[1] = j
                    break
            assert X[1] is not None and Y[0] is not None and Y[0] >= 0 and Y[1] >= 0
            NXr, NYr = X[1] - X[0] + 1, Y[1] - Y[0] + 1
            if NXD == 1:
                DLon_nk = 2.0 * PI / NXS
                DLon_n = DLon_nk
            else:
                DLon_nk = 2.0 * PI / NXD
                DLon_n = 2.0 * PI
            DLon_k = 2.0 * PI / NXD
            seg = [vD[jD - 1]] + [vS[Y[0] + j - 1] for j in range(1, NYr)] + [vD[jD]]
            Ak = (math.sin(vD[jD]) - math.sin(vD[jD - 1])) * DLon_k
            w1 = [DLon_nk * (math.sin(seg[j]) - math.sin(seg[j - 1])) / Ak for j in range(1, NYr + 1)]
            hh = lambda t: math.cos(t) + t * math.sin(t)
            for m in range(1, NXr + 1):
                for n in range(1, NYr + 1):
                    iS, jS = X[0] + m - 1, Y[0] + n - 1
                    if abs(w1[n - 1]) > 1e-14:
                        rows.append((iD - ISD + 1, jD - JSD + 1, iS - ISS + 1, jS - JSS + 1, w1[n - 1]))
                    if order > 1:
                        l1n, l2n = vS[Y[0] + n - 2], vS[Y[0] + n - 1]
                        An = (math.sin(l2n) - math.sin(l1n)) * DLon_n
                        w2 = (hh(seg[n]) - hh(seg[n - 1])) * DLon_nk / Ak - (hh(l2n) - hh(l1n)) * DLon_n * w1[n - 1] / An
                        if jS == JSS:
                            j1, j2 = jS, jS + 1
                        elif jS == JES:
                            j1, j2 = jS - 1, jS
                        else:
                            j1, j2 = jS - 1, jS + 1
                        DLat = yS[j2] - yS[j1]
                        if abs(w2) > 1e-14:
                            rows.append((iD - ISD + 1, jD - JSD + 1, iS - ISS + 1, j1 - JSS + 1, -w2 / DLat))
                            rows.append((iD - ISD + 1, jD - JSD + 1, iS - ISS + 1, j2 - JSS + 1, +w2 / DLat))
    a = np.array([r[:4] for r in rows], np.int32).reshape(-1, 4)
    w = np.array([r[4] for r in rows], np.float64)
    return a, w


def gaussian(I, J):
    mu, w = np.polynomial.legendre.leggauss(J)
    return 2.0 * np.pi * np.arange(I) / I, np.arcsin(mu), w


def make_j99():
    cases = {
        "refine_32x16_64x32": (gaussian(32, 16), gaussian(64, 32), 1),
        "coarsen_64x32_32x16": (gaussian(64, 32), gaussian(32, 16), 1),
        "identity_64x32": (gaussian(64, 32), gaussian(64, 32), 1),
        "zonal_dst_64x32_1x16": (gaussian(64, 32), (np.zeros(1), gaussian(1, 16)[1], gaussian(1, 16)[2]), 1),
        "order2_32x16_64x32": (gaussian(32, 16), gaussian(64, 32), 2),
    }
    out = {}
    for name, (S, D, order) in cases.items():
        a, w = j99_python(S[0], S[1], D[0], D[1], S[2], D[2], order)
        out[name + "_grid"] = np.concatenate([S[0], S[1], S[2], D[0], D[1], D[2]])
        out[name + "_shape"] = np.array([len(S[0]), len(S[1]), len(D[0]), len(D[1]), order], np.int64)
        out[name + "_idx"] = a
        out[name + "_w"] = w
    np.savez_compressed(os.path.join(OUT, "j99_small.npz"), **out)


# ---------------------------------------------------------------- SHT
def pbar_scipy(N, mu):
    """Pbar_n^m with integral Pbar^2 = 2, no Condon-Shortley phase (m-major)."""
    rows = []
    for m in range(N + 1):
        for n in range(m, N + 1):
            norm = math.sqrt((2 * n + 1) * math.factorial(n - m) / math.factorial(n + m))
            rows.append((-1) ** m * norm * lpmv(m, n, mu))
    return np.array(rows)


def make_sht():
    N, I, J, B = 21, 64, 32, 3
    mu, w = np.polynomial.legendre.leggauss(J)
    P = pbar_scipy(N, mu)
    rng = np.random.Generator(np.random.PCG64(11))
    nc = (N + 1) * (N + 2) // 2
    m_of = np.concatenate([np.full(N + 1 - m, m) for m in range(N + 1)])
    spec = rng.standard_normal((B, nc)) + 1j * rng.standard_normal((B, nc))
    spec[:, m_of == 0] = spec[:, m_of == 0].real
    # inverse: F_m(mu_j) over all latitudes, then a real inverse FFT
    grid = np.zeros((B, J, I))
    for b in range(B):
        F = np.zeros((J, I // 2 + 1), complex)
        for m in range(N + 1):
            sel = m_of == m
            F[:, m] = spec[b, sel] @ P[sel]
        F[:, 0] = F[:, 0].real
        grid[b] = np.fft.irfft(F, n=I, axis=1) * I
    # forward of that grid: G_m = rfft/I, s = 1/2 sum_j w_j Pbar G_m
    fwd = np.zeros((B, nc), complex)
    for b in range(B):
        G = np.fft.rfft(grid[b], axis=1) / I
        for m in range(N + 1):
            sel = m_of == m
            fwd[b, sel] = 0.5 * (P[sel] * w[None, :]) @ G[:, m]
    fwd[:, m_of == 0] = fwd[:, m_of == 0].real
    np.savez_compressed(os.path.join(OUT, "sht_t21.npz"), N=N, I=I, J=J, mu=mu, w=w, pbar=P,
                        spec=spec, grid=grid, fwd=fwd)


def implcpl_numpy(d, ih2o, consts):
    """SfcImplicitCoupling_VDiffForward (atm/dcpam_sfc_implicit_coupling_mod.f90:
    72-378) over whole levels at a time, Solve_TriDiagSystem_Forward
    (:380-405) on (kmax, ncol) arrays; every expression in the Fortran
    order."""
    G, Cp, R, DT = consts
    P, Tv, Z = d["Press"], d["VirTemp"], d["Height"]
    Ef, Eh = d["ExnerFull"], d["ExnerHalf"]
    K = P.shape[0] - 1
    ncol = P.shape[1]
    VTC = np.zeros((K + 1, ncol)); TTC = np.zeros((K + 1, ncol)); QTC = np.zeros((K + 1, ncol))
    for k in range(1, K):
        tmp = P[k] / (R * Tv[k]) / (Z[k] - Z[k - 1])  # Height(k+1) - Height(k), full levels 1-based
        VTC[k] = d["VelDiffCoef"][k] * tmp
        TTC[k] = d["TempDiffCoef"][k] * tmp
        QTC[k] = d["QMixDiffCoef"][k] * tmp

    def mat(TC):
        m = np.zeros((3, K, ncol))
        for k in range(1, K + 1):
            mass = -((P[k] - P[k - 1]) / G / (2.0 * DT))
            m[0, k - 1] = 0.0 if k == 1 else -TC[k - 1]
            m[1, k - 1] = mass + TC[k] if k == 1 else (mass + TC[k - 1] + TC[k] if k < K else mass + TC[k - 1])
            m[2, k - 1] = 0.0 if k == K else -TC[k]
        return m
    uv, qm = mat(VTC), mat(QTC)
    tm = np.zeros((3, K, ncol))
    for k in range(1, K + 1):
        mass = -(Cp * (P[k] - P[k - 1]) / G / (2.0 * DT))
        tm[0, k - 1] = 0.0 if k == 1 else -(Cp * Eh[k - 1] / Ef[k - 2] * TTC[k - 1])
        if k == 1:
            tm[1, k - 1] = mass + Cp * Eh[k] / Ef[k - 1] * TTC[k]
        elif k < K:
            tm[1, k - 1] = mass + Cp * Eh[k - 1] / Ef[k - 1] * TTC[k - 1] + Cp * Eh[k] / Ef[k - 1] * TTC[k]
        else:
            tm[1, k - 1] = mass + Cp * Eh[k - 1] / Ef[k - 1] * TTC[k - 1]
        tm[2, k - 1] = 0.0 if k == K else -(Cp * Eh[k] / Ef[k] * TTC[k])
    out = {"DUDt": -(d["MomFluxX"][1:] - d["MomFluxX"][:-1]), "DVDt": -(d["MomFluxY"][1:] - d["MomFluxY"][:-1]),
           "DTempDt": -(d["HeatFlux"][1:] - d["HeatFlux"][:-1]),
           "DQMixDt": -(d["QMixFlux"][:, 1:] - d["QMixFlux"][:, :-1])}
    C2 = np.stack([out["DUDt"][0], out["DVDt"][0], out["DTempDt"][0], out["DQMixDt"][ih2o - 1, 0]])

    def solve(m, r):
        with np.errstate(divide="ignore", invalid="ignore"):
            m[1, K - 1] = m[1, K - 1] / m[0, K - 1]
            r[K - 1] = r[K - 1] / m[0, K - 1]
            m[0, K - 1] = 1.0
            for k in range(K - 1, 0, -1):
                i = k - 1
                m[1, i] = (m[1, i] * m[1, i + 1] - m[2, i]) / (m[0, i] * m[1, i + 1])
                r[i] = (r[i] * m[1, i + 1] - m[2, i] * r[i + 1]) / (m[0, i] * m[1, i + 1])
                m[0, i] = 1.0
                m[2, i] = 0.0
    uvs = uv.copy()
    solve(uv, out["DUDt"])
    solve(uvs, out["DVDt"])
    solve(tm, out["DTempDt"])
    qs = qm.copy()
    for n in range(out["DQMixDt"].shape[0]):
        qm = qs.copy()
        solve(qm, out["DQMixDt"][n])
    Tmp = -((P[1] - P[0]) / G / (2.0 * DT))
    C1 = np.zeros((4, ncol))
    C1[0] = Tmp + VTC[1] - (-VTC[1]) / uv[1, 1]
    C2[0] = C2[0] - (-VTC[1]) * out["DUDt"][1] / uv[1, 1]
    C1[1] = Tmp + VTC[1] - (-VTC[1]) / uv[1, 1]
    C2[1] = C2[1] - (-VTC[1]) * out["DVDt"][1] / uv[1, 1]
    dt1 = Cp * Eh[1] * TTC[1] / Ef[0]
    dt2 = -(Cp * Eh[1] * TTC[1] / Ef[1])
    C1[2] = Cp * Tmp + dt1 - dt2 / tm[1, 1]
    C2[2] = C2[2] - dt2 * out["DTempDt"][1] / tm[1, 1]
    C1[3] = Tmp + QTC[1] - (-QTC[1]) / qm[1, 1]
    C2[3] = C2[3] - (-QTC[1]) * out["DQMixDt"][ih2o - 1, 1] / qm[1, 1]
    out.update(ImplCplCoef1=C1, ImplCplCoef2=C2, UVMtx=uv, TempMtx=tm, QMixMtx=qm)
    return out


def bilin_python(lonS, latS, lonR, latR):
    """gen_gridmapfile_lonlat2lonlat (common/grid_mapping_util.f90:32-182)
    transcribed line by line; north of the last source latitude (a read
    past the array in the reference) the last two source rows extrapolate,
    as the reference does south of the first."""
    nxs, nys, nxr, nyr = len(lonS), len(latS), len(lonR), len(latR)
    dlon_r, dlon_s = 360.0 / nxr, 360.0 / nxs
    rows = []
    for jr in range(1, nyr + 1):
        js, extp = None, True
        for j in range(1, nys):
            if latS[j - 1] < latR[jr - 1] <= latS[j]:
                js, extp = j, False
                break
        if extp:
            if latR[jr - 1] <= latS[0]:
                js = 1
            if latR[jr - 1] > latS[nys - 1]:
                js = nys
        if nxr == 1:
            if not extp:
                b1 = (latR[jr - 1] - latS[js - 1]) / (latS[js] - latS[js - 1])
                c1, c2 = (1.0 - b1) / nxs, b1 / nxs
                for i in range(1, nxs + 1):
                    rows += [(1, jr, i, js, c1), (1, jr, i, js % nys + 1, c2)]
            else:
                rows += [(1, jr, i, js, 1.0 / nxs) for i in range(1, nxs + 1)]
        elif nxs == 1:
            if not extp:
                b1 = (latR[jr - 1] - latS[js - 1]) / (latS[js] - latS[js - 1])
                for i in range(1, nxr + 1):
                    rows += [(i, jr, 1, js, 1.0 - b1), (i, jr, 1, js % nys + 1, b1)]
            else:
                rows += [(i, jr, 1, js, 1.0) for i in range(1, nxr + 1)]
        else:
            if extp and js == nys:
                js = nys - 1
            for ir in range(1, nxr + 1):
                i = int(dlon_r * (ir - 1) / dlon_s) + 1
                a1 = (lonR[ir - 1] - lonS[i - 1]) / (lonS[i % nxs] - lonS[i - 1])
                b1 = (latR[jr - 1] - latS[js - 1]) / (latS[js] - latS[js - 1])
                a2, b2 = 1.0 - a1, 1.0 - b1
                rows += [(ir, jr, i, js, a2 * b2), (ir, jr, i % nxs + 1, js, a1 * b2),
                         (ir, jr, i % nxs + 1, js % nys + 1, a1 * b1), (ir, jr, i, js % nys + 1, a2 * b1)]
    return rows


def xgrid_python(wA, wO):
    """generate_surface_exchage_grid (tool/gmapgen/gmapgen_main.f90:336-405)
    for JMA != JMO: merged latitude edges, Python's sorted() instead of the
    exchange sort."""
    JMA, JMO = len(wA), len(wO)
    FJA = [-math.pi / 2]
    for j in range(1, JMA + 1):
        FJA.append(math.asin(wA[j - 1] + math.sin(FJA[j - 1])))
    FJA[JMA] = math.pi / 2
    FJO = [-math.pi / 2]
    for j in range(1, JMO):
        FJO.append(math.asin(wO[j - 1] + math.sin(FJO[j - 1])))
    FJO.append(math.pi / 2)
    FJS = sorted(FJA[:JMA] + FJO[1:])
    lat, w = [], []
    for j in range(1, len(FJS)):
        wt = math.sin(FJS[j]) - math.sin(FJS[j - 1])
        if abs(wt) > 1e-12:
            lat.append(0.5 * (FJS[j - 1] + FJS[j]))
            w.append(wt)
    return np.array(lat), np.array(w)


def make_bilin():
    out = {}
    cases = {"t21_to_t42": (gaussian(64, 32), gaussian(128, 64)),
             "t42_to_t21": (gaussian(128, 64), gaussian(64, 32)),
             "t21_to_reg": (gaussian(64, 32), regular(72, 36)),
             "axi_dst": (gaussian(64, 32), (np.zeros(1), regular(1, 20)[1])),
             "axi_src": ((np.zeros(1), regular(1, 16)[1]), gaussian(64, 32))}
    for name, (S, R) in cases.items():
        rows = bilin_python(S[0], S[1], R[0], R[1])
        out[name + "_grid"] = np.array([len(S[0]), len(S[1]), len(R[0]), len(R[1])])
        out[name + "_lon_lat"] = np.concatenate([S[0], S[1], R[0], R[1]])
        out[name + "_idx"] = np.array([r[:4] for r in rows], dtype=np.int32)
        out[name + "_w"] = np.array([r[4] for r in rows], dtype=np.float64)
    lat, w = xgrid_python(list(gaussian(64, 32)[2]), list(regular_w(64)))
    out["xgrid_lat"], out["xgrid_w"] = lat, w
    np.savez_compressed(os.path.join(OUT, "bilin_small.npz"), **out)


def regular(nx, ny):
    """Cell-centred regular grid (lon from 0, lat S to N) in radians."""
    lon = 2.0 * np.pi * np.arange(nx) / nx
    e = np.linspace(-np.pi / 2, np.pi / 2, ny + 1)
    return lon, 0.5 * (e[:-1] + e[1:])


def regular_w(ny):
    e = np.linspace(-np.pi / 2, np.pi / 2, ny + 1)
    return np.sin(e[1:]) - np.sin(e[:-1])


def make_implcpl():
    import importlib
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(OUT)))
    synth = importlib.import_module("dennou-ccm_gb300.synth")
    d = synth.column_profiles(24, 12, ncmax=2, seed=5)
    o = implcpl_numpy(d, 1, synth.IMPLCPL_CONSTS)
    np.savez_compressed(os.path.join(OUT, "implcpl_small.npz"), consts=np.array(synth.IMPLCPL_CONSTS), ih2o=1,
                        **{"in_" + k: v for k, v in d.items()}, **{"out_" + k: v for k, v in o.items()})


def spec_numpy(N, kind, spec, a, order, tau, dt, corr):
    n = np.array([nn for m in range(N + 1) for nn in range(m, N + 1)], dtype=np.float64)
    nn = n * (n + 1)
    if kind == 0:
        f = -nn / a ** 2
    elif kind == 1:
        f = np.where(n == 0, 0.0, -(a ** 2) / np.where(n == 0, 1.0, nn))
    else:
        p = order // 2
        K = np.power(nn, p) / a ** (2 * p)
        c = 2.0 ** p / a ** (2 * p) if corr else 0.0
        nu = 1.0 / (tau * (np.power(N * (N + 1.0), p) / a ** (2 * p) - c))
        D = np.where(n == 0, 0.0, nu * (K - c))
        f = -D if kind == 2 else 1.0 / (1.0 + dt * D)
    return spec * f[None, :]


def make_spec():
    N, a, order, tau, dt = 21, 6.371e6, 8, 3 * 3600.0, 1200.0
    rng = np.random.Generator(np.random.PCG64(11))
    nc = (N + 1) * (N + 2) // 2
    spec = rng.standard_normal((3, nc)) + 1j * rng.standard_normal((3, nc))
    out = {"N": N, "a": a, "order": order, "tau": tau, "dt": dt, "spec": spec}
    for kind in range(4):
        for corr in (0, 1):
            out["out_%d_%d" % (kind, corr)] = spec_numpy(N, kind, spec, a, order, tau, dt, corr)
    np.savez_compressed(os.path.join(OUT, "spec_ops_t21.npz"), **out)


if __name__ == "__main__":
    make_spec()
    make_flux()
    make_j99()
    make_sht()
    make_implcpl()
    make_bilin()
    for f in sorted(os.listdir(OUT)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(OUT, f)))
