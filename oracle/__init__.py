"""ctypes bindings of the CPU oracle (test infrastructure only).

The oracle is what the GPU results are compared against: tests,
``__graft_entry__.smoke()`` and the CPU baseline of ``bench.py`` call it;
the product library never does.  See
``oracle.h`` for what each function restates and why parity is unpinned.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "liboracle.so")
_lib = None

FLUX_ARGS = [
    "WindStressX", "WindStressY", "SenHFlx", "QVapMFlx", "LatHFlx",
    "SfcVelTransCoef", "SfcTempTransCoef", "SfcQVapTransCoef",
    "DelVarImplCPL", "SUwRFlx", "LUwRFlx", "SfcHFlx_ns", "SfcHFlx_sr",
    "DSfcHFlxDTs", "WindU", "WindV", "SfcAirTemp", "QVap1", "SDwRFlx",
    "LDwRFlx", "ImplCplCoef1", "ImplCplCoef2", "SfcTemp", "SfcAlbedo",
    "SIceCon", "a_Sig1Info", "SfcHeight", "SfcPress",
]


def build(force=False):
    """Compile liboracle.so with make (gcc, FP64, OpenMP)."""
    if force or not os.path.exists(_LIB_PATH):
        subprocess.check_call(["make", "-s", "-C", _HERE, "-B" if force else "liboracle.so"])
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        P = ctypes.c_void_p
        i32, i64, f64 = ctypes.c_int, ctypes.c_int64, ctypes.c_double
        L.oracle_sfc_bulk_flux.argtypes = [P, i32, i32, i32, i32, i32, i32]
        L.oracle_j99_gen.argtypes = [P, i32, P, i32, P, i32, P, i32, P, P, i32, i32,
                                     i64, P, P, P, P, P, P]
        L.oracle_j99_gen.restype = i32
        L.oracle_table_to_index.argtypes = [i64, P, P, P, P, i32, i32, P, P]
        L.oracle_remap_apply.argtypes = [i64, P, P, P, i64, P, i64, P, i32]
        L.oracle_remap_apply.restype = i32
        L.oracle_area_integral.argtypes = [i64, P, P]
        L.oracle_area_integral.restype = f64
        L.oracle_gauss_nodes.argtypes = [i32, P, P]
        L.oracle_pnm.argtypes = [i32, i32, P, P]
        L.oracle_sht_inverse.argtypes = [i32, i32, i32, i32, P, P]
        L.oracle_sht_forward.argtypes = [i32, i32, i32, i32, P, P]
        L.oracle_rfft_row.argtypes = [i32, P, i32, P]
        L.oracle_implcpl_forward.argtypes = [P, P, P, P, P, i64, i32, i32, i32, P]
        L.oracle_implcpl_backward.argtypes = [P, P, P, P, P, P, P, i64, i32, i32, f64]
        L.oracle_bilin_gen.argtypes = [P, i32, P, i32, P, i32, P, i32, i64, P, P, P, P, P, P]
        L.oracle_bilin_gen.restype = i32
        L.oracle_exchange_grid_lat.argtypes = [P, P, i32, P, P, i32, P, P]
        L.oracle_exchange_grid_lat.restype = i32
        L.oracle_spec_apply.argtypes = [i32, i32, f64, i32, f64, f64, i32, i32, P, P]
        L.oracle_spec_apply.restype = i32
        L.oracle_set_threads.argtypes = [i32]
        L.oracle_get_threads.restype = i32
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def set_threads(n):
    lib().oracle_set_threads(int(n))


def get_threads():
    return int(lib().oracle_get_threads())


# ------------------------------------------------------------------ flux
def sfc_bulk_flux(arrays, IA, JA, IS, IE, JS, JE):
    """arrays: dict name -> Fortran-ordered float64 array (modified in place)."""
    ptrs = (ctypes.c_void_p * len(FLUX_ARGS))()
    for k, name in enumerate(FLUX_ARGS):
        a = arrays[name]
        assert a.dtype == np.float64 and (a.flags.f_contiguous or a.ndim == 1)
        ptrs[k] = a.ctypes.data
    lib().oracle_sfc_bulk_flux(ctypes.cast(ptrs, ctypes.c_void_p), IA, JA, IS, IE, JS, JE)


# ----------------------------------------------------------------- remap
def j99_gen(lonS, latS, lonD, latD, latwtS, latwtD, order=1, mode=0):
    """Rows (iD, jD, iS, jS, w) of the Jones-99 table in the reference's order."""
    args = [np.ascontiguousarray(x, dtype=np.float64) for x in (lonS, latS, lonD, latD, latwtS, latwtD)]
    lonS, latS, lonD, latD, latwtS, latwtD = args
    cap = 0
    nrow = ctypes.c_int64(0)
    while True:
        bufs = [np.zeros(max(cap, 1), np.int32) for _ in range(4)] + [np.zeros(max(cap, 1), np.float64)]
        st = lib().oracle_j99_gen(_p(lonS), len(lonS), _p(latS), len(latS), _p(lonD), len(lonD),
                                  _p(latD), len(latD), _p(latwtS), _p(latwtD), int(order), int(mode),
                                  cap, *[_p(b) for b in bufs], ctypes.byref(nrow))
        if st < 0:
            raise RuntimeError("oracle_j99_gen: search failed (%d)" % st)
        if st == 0:
            n = nrow.value
            return tuple(b[:n] for b in bufs)
        cap = nrow.value


def table_to_index(iD, jD, iS, jS, GNXS, GNXR):
    n = len(iD)
    send = np.zeros(n, np.int32)
    recv = np.zeros(n, np.int32)
    c = [np.ascontiguousarray(x, dtype=np.int32) for x in (iD, jD, iS, jS)]
    lib().oracle_table_to_index(n, *[_p(x) for x in c], GNXS, GNXR, _p(send), _p(recv))
    return send, recv


def remap_apply(send_index, recv_index, coef, send, rn1):
    """send: (sn1, nd) Fortran order.  Returns recv (rn1, nd) Fortran order."""
    send = np.asfortranarray(send, dtype=np.float64)
    sn1, nd = send.shape
    recv = np.zeros((rn1, nd), np.float64, order="F")
    si = np.ascontiguousarray(send_index, np.int32)
    ri = np.ascontiguousarray(recv_index, np.int32)
    cf = np.ascontiguousarray(coef, np.float64)
    st = lib().oracle_remap_apply(len(si), _p(si), _p(ri), _p(cf), sn1, _p(send), rn1, _p(recv), nd)
    if st != 0:
        raise ValueError("index out of range")
    return recv


def area_integral(f, area):
    f = np.ascontiguousarray(f, np.float64).ravel()
    area = np.ascontiguousarray(area, np.float64).ravel()
    return lib().oracle_area_integral(len(f), _p(f), _p(area))


# ------------------------------------------------------------------- SHT
def ncoef(N):
    return (N + 1) * (N + 2) // 2


def gauss_nodes(J):
    mu = np.zeros(J)
    w = np.zeros(J)
    lib().oracle_gauss_nodes(J, _p(mu), _p(w))
    return mu, w


def pnm(N, J):
    mu, _ = gauss_nodes(J)
    p = np.zeros(ncoef(N) * J)
    lib().oracle_pnm(N, J, _p(mu), _p(p))
    return p.reshape(ncoef(N), J)


def sht_inverse(N, I, J, spec):
    """spec: complex128 [batch, ncoef] -> grid float64 [batch, J, I]."""
    spec = np.ascontiguousarray(spec, np.complex128)
    B = spec.shape[0]
    grid = np.zeros((B, J, I))
    lib().oracle_sht_inverse(N, I, J, B, _p(spec), _p(grid))
    return grid


def sht_forward(N, I, J, grid):
    grid = np.ascontiguousarray(grid, np.float64)
    B = grid.shape[0]
    spec = np.zeros((B, ncoef(N)), np.complex128)
    lib().oracle_sht_forward(N, I, J, B, _p(grid), _p(spec))
    return spec


def rfft_row(g, M):
    g = np.ascontiguousarray(g, np.float64)
    out = np.zeros(M, np.complex128)
    lib().oracle_rfft_row(len(g), _p(g), M, _p(out))
    return out


# ------------------------------------------------------ implicit coupling
IMPLCPL_IN = ["MomFluxX", "MomFluxY", "HeatFlux", "QMixFlux", "Press", "ExnerFull", "ExnerHalf",
              "VirTemp", "Height", "VelDiffCoef", "TempDiffCoef", "QMixDiffCoef"]
IMPLCPL_OUT = ["DUDt", "DVDt", "DTempDt", "DQMixDt", "ImplCplCoef1", "ImplCplCoef2"]


def implcpl_forward(prof, ih2o, consts):
    """SfcImplicitCoupling_VDiffForward over the columns of prof (arrays
    [k][c], tracers [n][k][c], as synth.column_profiles returns them).
    Returns the outputs (DUDt, DVDt, DTempDt [kmax][c], DQMixDt [n][kmax][c],
    ImplCplCoef1/2 [4][c]) and the eliminated matrices UVMtx, TempMtx,
    QMixMtx [3][kmax][c] (sub-, main, super-diagonal)."""
    arrs = [np.ascontiguousarray(prof[n], dtype=np.float64) for n in IMPLCPL_IN]
    kmax1, ncol = arrs[0].shape
    kmax = kmax1 - 1
    ncmax = arrs[3].shape[0]
    out = {"DUDt": np.zeros((kmax, ncol)), "DVDt": np.zeros((kmax, ncol)), "DTempDt": np.zeros((kmax, ncol)),
           "DQMixDt": np.zeros((ncmax, kmax, ncol)), "ImplCplCoef1": np.zeros((4, ncol)),
           "ImplCplCoef2": np.zeros((4, ncol))}
    mats = {n: np.zeros((3, kmax, ncol)) for n in ("UVMtx", "TempMtx", "QMixMtx")}
    pin = (ctypes.c_void_p * len(arrs))(*[a.ctypes.data for a in arrs])
    pout = (ctypes.c_void_p * len(IMPLCPL_OUT))(*[out[n].ctypes.data for n in IMPLCPL_OUT])
    c = np.ascontiguousarray(consts, dtype=np.float64)
    lib().oracle_implcpl_forward(ctypes.cast(pin, ctypes.c_void_p), ctypes.cast(pout, ctypes.c_void_p),
                                 _p(mats["UVMtx"]), _p(mats["TempMtx"]), _p(mats["QMixMtx"]), ncol, kmax,
                                 ncmax, int(ih2o), _p(c))
    out.update(mats)
    return out


def implcpl_backward(mats, tend, DelTime):
    """SfcImplicitCoupling_VDiffBackward on copies of the tendencies (dict
    with DUDt, DVDt, DTempDt, DQMixDt) with the matrices of the forward."""
    t = {n: np.array(tend[n], dtype=np.float64, order="C") for n in ("DUDt", "DVDt", "DTempDt", "DQMixDt")}
    m = [np.ascontiguousarray(mats[n], dtype=np.float64) for n in ("UVMtx", "TempMtx", "QMixMtx")]
    kmax, ncol = t["DUDt"].shape
    ncmax = t["DQMixDt"].shape[0]
    lib().oracle_implcpl_backward(*[_p(x) for x in m], _p(t["DUDt"]), _p(t["DVDt"]), _p(t["DTempDt"]),
                                  _p(t["DQMixDt"]), ncol, kmax, ncmax, float(DelTime))
    return t


# -------------------------------------------- bilinear table, exchange grid
def bilin_gen(lonS, latS, lonR, latR):
    """Rows (iR, jR, iS, jS, w) of the bilinear table in the reference's
    order (north of the last source latitude: linear extrapolation from the
    last two; ValueError if the source has a single latitude)."""
    a = [np.ascontiguousarray(x, dtype=np.float64) for x in (lonS, latS, lonR, latR)]
    cap = 0
    nrow = ctypes.c_int64(0)
    while True:
        bufs = [np.zeros(max(cap, 1), np.int32) for _ in range(4)] + [np.zeros(max(cap, 1), np.float64)]
        st = lib().oracle_bilin_gen(_p(a[0]), len(a[0]), _p(a[1]), len(a[1]), _p(a[2]), len(a[2]), _p(a[3]),
                                    len(a[3]), cap, *[_p(b) for b in bufs], ctypes.byref(nrow))
        if st < 0:
            raise ValueError("oracle_bilin_gen: no source latitude pair (%d)" % st)
        if st == 0:
            return tuple(b[:nrow.value] for b in bufs)
        cap = nrow.value


def exchange_grid_lat(latA, wA, latO, wO):
    """Latitudes and sin-latitude widths of the surface exchange grid."""
    a = [np.ascontiguousarray(x, dtype=np.float64) for x in (latA, wA, latO, wO)]
    n = len(a[0]) + len(a[2])
    lat, w = np.zeros(n), np.zeros(n)
    m = lib().oracle_exchange_grid_lat(_p(a[0]), _p(a[1]), len(a[0]), _p(a[2]), _p(a[3]), len(a[2]),
                                       _p(lat), _p(w))
    return lat[:m], w[:m]



# --------------------------------------------------- spectral operators
SPEC_LAPLACIAN, SPEC_INV_LAPLACIAN, SPEC_HDIFF_TENDENCY, SPEC_HDIFF_IMPLICIT = 0, 1, 2, 3


def spec_apply(N, kind, spec, radius, order=8, efold_time=1.0, dt=0.0, rotation_correction=False):
    """complex128 [batch, ncoef] -> the same scaled per total wavenumber."""
    spec = np.ascontiguousarray(spec, np.complex128)
    out = np.zeros_like(spec)
    rc = lib().oracle_spec_apply(N, kind, radius, order, efold_time, dt, int(bool(rotation_correction)),
                                 spec.shape[0], _p(spec), _p(out))
    if rc != 0:
        raise ValueError("oracle_spec_apply: invalid parameters")
    return out
