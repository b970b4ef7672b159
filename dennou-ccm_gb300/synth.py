"""Seeded synthetic inputs of the coupling-step workloads.

The reference publishes no benchmark data, so inputs are generated with the
shapes and value distributions of the five workloads:

* spectra: complex Gaussian, variance proportional to n**-3 for n >= 1, the
  n = 0 mode zero, imaginary part zero for m = 0 (numpy PCG64, seed per
  member);
* surface state per ocean column: SST = 273 + 27 cos^2(lat) K, air
  temperature SST - 2 K + U(-1, 1) K, specific humidity at 80 % of the
  reference's own saturation formula
  (sfc/DSFCM_Util_SfcBulkFlux_mod.f90:211-212), wind components N(0, 5 m/s),
  surface pressure 1e5 Pa * (1 + U(-0.01, 0.01)), no sea ice, ice-slot
  temperature 271.35 K, albedo 0.06 (ocean) / 0.5 (ice), shortwave
  300 max(cos lat, 0) W m-2, longwave 0.8 sigma T_air^4, surface height 0
  (as sfc/dccm_sfc_mod.f90:885), a_Sig1Info = (0.995, 0.01), and
  implicit-coupling coefficients ps*dsigma/(g*2*dt) (Cp times that for
  temperature), dt = 1200 s, ImplCplCoef2 = 0;
* land mask: Bernoulli(0.3) per cell.
"""
import numpy as np

GRAV = 9.8
CP = 1616.0
STB = 5.670373e-8
GASR_WET = 8.3144621 / 1.8e-2


def ncoef(N):
    return (N + 1) * (N + 2) // 2


def gaussian_axes(I, J):
    """Longitudes 2 pi i / I and Gaussian latitudes ascending, with weights."""
    mu, w = np.polynomial.legendre.leggauss(J)
    return 2.0 * np.pi * np.arange(I) / I, np.arcsin(mu), np.full(I, 2.0 * np.pi / I), w


def regular_axes(I, J):
    """Cell-centred regular lon-lat grid (e.g. 1 degree: I=360, J=180)."""
    lon = np.deg2rad((np.arange(I) + 0.5) * 360.0 / I)
    e = np.deg2rad(-90.0 + 180.0 * np.arange(J + 1) / J)
    lat = 0.5 * (e[1:] + e[:-1])
    return lon, lat, np.full(I, 2.0 * np.pi / I), np.sin(e[1:]) - np.sin(e[:-1])


def spectra(N, batch, seed=0):
    """complex128 [batch, ncoef]: variance n**-3, n=0 zero, Im = 0 for m = 0."""
    rng = np.random.Generator(np.random.PCG64(seed))
    nc = ncoef(N)
    n_of = np.concatenate([np.arange(m, N + 1) for m in range(N + 1)])
    m_of = np.concatenate([np.full(N + 1 - m, m) for m in range(N + 1)])
    sd = np.where(n_of >= 1, np.maximum(n_of, 1).astype(np.float64) ** -1.5, 0.0) / np.sqrt(2.0)
    s = (rng.standard_normal((batch, nc)) + 1j * rng.standard_normal((batch, nc))) * sd
    s[:, m_of == 0] = s[:, m_of == 0].real * np.sqrt(2.0)
    return s


def qsat(T, ps):
    """The reference's saturation specific humidity (EpsV = 1)."""
    return 1.0 * 611.0 / ps * np.exp(2425300.0 / GASR_WET * (1.0 / 273.0 - 1.0 / T))


def surface_state(lat, nx, seed=0, sea_ice=None, sig1=(0.995, 0.01), dt=1200.0, halo_fill=np.nan):
    """Dict of Fortran-ordered (IA, JA[, k]) arrays with a halo of 1 for the
    bulk flux on an nx x len(lat) grid (lon fastest)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    ny = len(lat)
    IA, JA = nx + 2, ny + 2
    coslat = np.cos(lat)[None, :] * np.ones((nx, 1))
    sst = 273.0 + 27.0 * coslat ** 2
    ta = sst - 2.0 + rng.uniform(-1.0, 1.0, (nx, ny))
    ps = 1e5 * (1.0 + rng.uniform(-0.01, 0.01, (nx, ny)))
    u = rng.normal(0.0, 5.0, (nx, ny))
    v = rng.normal(0.0, 5.0, (nx, ny))
    q = 0.8 * qsat(ta, ps)
    ice = np.zeros((nx, ny)) if sea_ice is None else sea_ice
    c1 = ps * sig1[1] / (GRAV * 2.0 * dt)

    def f2(x):
        a = np.full((IA, JA), halo_fill, order="F")
        a[1:-1, 1:-1] = x
        return a

    def f3(xs):
        a = np.full((IA, JA, len(xs)), halo_fill, order="F")
        for k, x in enumerate(xs):
            a[1:-1, 1:-1, k] = x
        return a

    d = {
        "WindU": f2(u), "WindV": f2(v), "SfcAirTemp": f2(ta), "QVap1": f2(q),
        "SDwRFlx": f2(300.0 * np.maximum(coslat, 0.0)), "LDwRFlx": f2(0.8 * STB * ta ** 4),
        "ImplCplCoef1": f3([c1, c1, CP * c1, c1]), "ImplCplCoef2": f3([0 * c1] * 4),
        "SfcTemp": f3([sst, np.full((nx, ny), 271.35), np.zeros((nx, ny))]),
        "SfcAlbedo": f3([np.full((nx, ny), 0.06), np.full((nx, ny), 0.5), np.zeros((nx, ny))]),
        "SIceCon": f2(ice), "a_Sig1Info": np.array(sig1, np.float64),
        "SfcHeight": f2(np.zeros((nx, ny))), "SfcPress": f2(ps),
    }
    return d, (IA, JA, 2, IA - 1, 2, JA - 1)


def flux_outputs(IA, JA, fill=np.nan):
    """Output arrays of the bulk flux, pre-filled (to detect untouched cells)."""
    out = {}
    for n in ("WindStressX", "WindStressY", "SenHFlx", "QVapMFlx", "LatHFlx", "SfcVelTransCoef",
              "SfcTempTransCoef", "SfcQVapTransCoef", "SUwRFlx", "LUwRFlx", "SfcHFlx_ns",
              "SfcHFlx_sr", "DSfcHFlxDTs"):
        out[n] = np.full((IA, JA, 3), fill, order="F")
    out["DelVarImplCPL"] = np.full((IA, JA, 4), fill, order="F")
    return out


def land_mask(nx, ny, frac=0.3, seed=0):
    """uint8 (ny, nx) flattened lon-fastest: 1 = ocean, 0 = land."""
    rng = np.random.Generator(np.random.PCG64(seed))
    return (rng.uniform(size=nx * ny) >= frac).astype(np.uint8)


# Constants of the implicit-coupling inputs (DCPAM defaults): Grav, CpDry,
# GasRDry, and the 1200 s step of the T21L16 coupled configuration.
IMPLCPL_CONSTS = (9.8, 1004.6, 287.04, 1200.0)


def column_profiles(ncol, kmax, ncmax=1, seed=0):
    """Atmosphere columns for the implicit surface coupling: half levels
    (kmax+1, ncol) k = 0 (surface) .. kmax (top, p = 0), full levels
    (kmax, ncol), tracer fluxes (ncmax, kmax+1, ncol); row-major [k][c] is
    the reference's (i, j, k) layout with the columns flattened.  Sigma
    levels, a dry-adiabat-like temperature, hydrostatic heights, diffusion
    coefficients decaying over 1 km and surface fluxes decaying likewise
    (seeded PCG64)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    G, Cp, R, _ = IMPLCPL_CONSTS
    kappa = R / Cp
    sh = 1.0 - (np.arange(kmax + 1) / kmax) ** 1.5           # sigma at half levels, 1 -> 0
    sf = 0.5 * (sh[:-1] + sh[1:])                              # full levels
    ps = 1.0e5 * (1.0 + rng.uniform(-0.02, 0.02, ncol))
    ph = sh[:, None] * ps[None, :]
    pf = sf[:, None] * ps[None, :]
    tf = 288.0 * sf[:, None] ** 0.19 + rng.uniform(-1.0, 1.0, (kmax, ncol))
    th = np.empty((kmax + 1, ncol))
    th[0] = tf[0] + 1.0
    th[1:kmax] = 0.5 * (tf[:-1] + tf[1:])
    th[kmax] = tf[-1]
    zf = R * tf / G * np.log(1.0 / sf[:, None])
    zh = np.empty((kmax + 1, ncol))
    zh[0] = 0.0
    zh[1:kmax] = 0.5 * (zf[:-1] + zf[1:])
    zh[kmax] = zf[-1] + (zf[-1] - zf[-2])
    decay = np.exp(-zh / 1000.0)
    kv = (10.0 * decay + 0.1) * rng.uniform(0.5, 1.5, ncol)[None, :]
    kv[0] = kv[kmax] = 0.0
    taux = rng.normal(0.0, 0.1, ncol)
    tauy = rng.normal(0.0, 0.1, ncol)
    heat = rng.normal(20.0, 10.0, ncol)
    qflx = np.abs(rng.normal(3e-5, 1e-5, (ncmax, ncol)))
    mom_x, mom_y, hflx = taux[None] * decay, tauy[None] * decay, heat[None] * decay
    for a in (mom_x, mom_y, hflx):
        a[kmax] = 0.0
    qf = qflx[:, None, :] * decay[None]
    qf[:, kmax] = 0.0
    return {"MomFluxX": mom_x, "MomFluxY": mom_y, "HeatFlux": hflx, "QMixFlux": qf,
            "Press": ph, "ExnerFull": (pf / 1.0e5) ** kappa, "ExnerHalf": (ph / 1.0e5) ** kappa,
            "VirTemp": th, "Height": zf, "VelDiffCoef": kv, "TempDiffCoef": 1.2 * kv,
            "QMixDiffCoef": 1.1 * kv}
