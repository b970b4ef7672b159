"""Host-side Python mirror of the dccm_gb300 C ABI.

The product is the C-ABI library ``libdccm_gb300.so`` (CUDA kernels for
sm_103a behind ``include/dccm_gb300.h``).  This module loads it with ctypes
and exposes the reference's procedure names with the reference's argument
meaning, so that tests and the benchmark read like calls into the Fortran
modules they replace:

* ``DSFCM_Util_SfcBulkFlux_Get`` (sfc/DSFCM_Util_SfcBulkFlux_mod.f90:108-151)
* ``gen_gridmapfile_lonlat2lonlat`` and ``set_mappingTable_interpCoef``
  (common/grid_mapping_util_jones99.f90:35-41, :446-462)
* ``RemapPlan`` / ``interpolate_data`` (common/interpolation_data_latlon_mod.f90:116-306,
  common/interpolate_data.f90:1-15)
* ``ShtPlan`` (SPML w_Initial + transforms, tool/gmapgen/gmapgen_main.f90:262-305)

There is no fallback: if the library is missing or cannot be loaded every
call raises.  Errors from the library (negative status codes) raise
``DccmError``.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libdccm_gb300.so")

FLUX_ARGS = [
    "WindStressX", "WindStressY", "SenHFlx", "QVapMFlx", "LatHFlx",
    "SfcVelTransCoef", "SfcTempTransCoef", "SfcQVapTransCoef",
    "DelVarImplCPL", "SUwRFlx", "LUwRFlx", "SfcHFlx_ns", "SfcHFlx_sr",
    "DSfcHFlxDTs", "WindU", "WindV", "SfcAirTemp", "QVap1", "SDwRFlx",
    "LDwRFlx", "ImplCplCoef1", "ImplCplCoef2", "SfcTemp", "SfcAlbedo",
    "SIceCon", "a_Sig1Info", "SfcHeight", "SfcPress",
]
FLUX_OUT = FLUX_ARGS[:14]
FLUX_IN = FLUX_ARGS[14:]
FLUX_SLOTS = {n: 3 for n in FLUX_OUT}
FLUX_SLOTS.update({"DelVarImplCPL": 4, "ImplCplCoef1": 4, "ImplCplCoef2": 4,
                   "SfcTemp": 3, "SfcAlbedo": 3})

J99_REF, J99_CONSERVE = 0, 1
SHT_FP64, SHT_MIXED, SHT_MIXED_FP16 = 0, 1, 2


class DccmError(RuntimeError):
    def __init__(self, status, what=""):
        self.status = status
        msg = _lib.dccm_status_string(status).decode() if _lib is not None else str(status)
        super().__init__("%s: %s (status %d, cuda %d)" % (what, msg, status,
                                                          _lib.dccm_last_cuda_error() if _lib else 0))


class FluxArgs(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in FLUX_ARGS]


class SfcGrid(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in ("IA", "JA", "IS", "IE", "JS", "JE")]


IMPLCPL_FWD_ARGS = ["xyr_MomFluxX", "xyr_MomFluxY", "xyr_HeatFlux", "xyrf_QMixFlux", "xyr_Press",
                    "xyz_Exner", "xyr_Exner", "xyr_VirTemp", "xyz_Height", "xyr_VelDiffCoef",
                    "xyr_TempDiffCoef", "xyr_QMixDiffCoef", "xyz_DUDt", "xyz_DVDt", "xyz_DTempDt",
                    "xyzf_DQMixDt", "xya_ImplCplCoef1", "xya_ImplCplCoef2"]


class ImplCplConsts(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in ("Grav", "CpDry", "GasRDry", "DelTime")]


class ImplCplForwardArgs(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in IMPLCPL_FWD_ARGS]


_lib = None
_SIGS = {
    "dccm_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "dccm_abi_version": (ctypes.c_int, []),
    "dccm_last_cuda_error": (ctypes.c_int, []),
    "dccm_sfc_bulk_flux_get": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "dccm_sfc_bulk_flux_get_dev": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "dccm_bilinear_generate": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                                              ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                                              ctypes.c_void_p, ctypes.c_void_p]),
    "dccm_exchange_grid": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                          ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.c_void_p]),
    "dccm_implcpl_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                           ctypes.c_void_p, ctypes.c_void_p]),
    "dccm_implcpl_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "dccm_implcpl_forward": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "dccm_implcpl_forward_dev": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "dccm_implcpl_backward": (ctypes.c_int, [ctypes.c_void_p] * 5),
    "dccm_implcpl_backward_dev": (ctypes.c_int, [ctypes.c_void_p] * 6),
    "dccm_implcpl_matrices": (ctypes.c_int, [ctypes.c_void_p] * 4),
    "dccm_implcpl_info": (ctypes.c_int, [ctypes.c_void_p] * 4),
    "dccm_j99_generate": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                                         ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                                         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                         ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]),
    "dccm_remap_table_size": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "dccm_remap_table_rows": (ctypes.c_int, [ctypes.c_void_p] * 6),
    "dccm_remap_table_write": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p]),
    "dccm_remap_table_read": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_void_p]),
    "dccm_remap_table_index": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                              ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "dccm_remap_table_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "dccm_remap_plan_create": (ctypes.c_int, [ctypes.c_int64, ctypes.c_int64, ctypes.c_int64,
                                              ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                              ctypes.c_void_p]),
    "dccm_remap_plan_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "dccm_remap_plan_info": (ctypes.c_int, [ctypes.c_void_p] * 4),
    "dccm_interpolate_data": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p,
                                             ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int]),
    "dccm_remap_apply_dev": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                            ctypes.c_int64, ctypes.c_int, ctypes.c_void_p]),
    "dccm_area_integral_dev": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                              ctypes.c_void_p, ctypes.c_void_p]),
    "dccm_area_integral_noalloc_dev": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                                      ctypes.c_void_p, ctypes.c_void_p]),
    "dccm_sht_plan_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                            ctypes.c_int, ctypes.c_void_p]),
    "dccm_sht_plan_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "dccm_sht_axes": (ctypes.c_int, [ctypes.c_void_p] * 5),
    "dccm_sht_gauss": (ctypes.c_int, [ctypes.c_void_p] * 3),
    "dccm_sht_pnm": (ctypes.c_int, [ctypes.c_void_p] * 2),
    "dccm_sht_inverse_dev": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                            ctypes.c_void_p]),
    "dccm_sht_forward_dev": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                            ctypes.c_void_p]),
    "dccm_sht_inverse": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]),
    "dccm_sht_forward": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]),
    "dccm_sht_status": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "dccm_sht_xya_wa_dev": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                           ctypes.c_void_p]),
    "dccm_sht_wa_xya_dev": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                           ctypes.c_void_p]),
    "dccm_sht_xya_wa": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]),
    "dccm_sht_wa_xya": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]),
    "dccm_sht_spec_from_wa_dev": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                 ctypes.c_int, ctypes.c_void_p]),
    "dccm_sht_wa_from_spec_dev": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                 ctypes.c_int, ctypes.c_void_p]),
    "dccm_sht_ensemble_create": (ctypes.c_int, [ctypes.c_int] + [ctypes.c_void_p] * 4 + [ctypes.c_int,
                                                                                     ctypes.c_void_p]),
    "dccm_sht_ensemble_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "dccm_sht_ensemble_inverse_dev": (ctypes.c_int, [ctypes.c_void_p] * 5),
    "dccm_sht_ensemble_forward_dev": (ctypes.c_int, [ctypes.c_void_p] * 5),
    "dccm_sht_ensemble_status": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "dccm_sht_ensemble_groups": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "dccm_step_autotune": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_void_p]),
    "dccm_tune_set": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int]),
    "dccm_tune_get": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_void_p]),
    "dccm_step_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "dccm_step_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "dccm_step_run": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "dccm_step_run_timed": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "dccm_step_run_host": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                          ctypes.c_void_p, ctypes.c_int]),
    "dccm_step_launch_host": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                             ctypes.c_void_p, ctypes.c_int]),
    "dccm_step_host_choice": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "dccm_step_host_release": (ctypes.c_int, [ctypes.c_void_p]),
    "dccm_fp64_peak": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "dccm_fp64_fn_dev": (ctypes.c_int, [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                        ctypes.c_void_p]),
    "dccm_spec_apply": (ctypes.c_int, [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.c_int]),
    "dccm_spec_apply_dev": (ctypes.c_int, [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.c_int, ctypes.c_void_p]),
    "dccm_step_autotune_host": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                               ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]),
}


class StepRemap(ctypes.Structure):
    _fields_ = [("plan", ctypes.c_void_p), ("nfields", ctypes.c_int), ("src", ctypes.c_void_p),
                ("ld_src", ctypes.c_int64), ("dst", ctypes.c_void_p), ("ld_dst", ctypes.c_int64),
                ("nsub", ctypes.c_int), ("ld_dst2", ctypes.c_int64)]


class StepDesc(ctypes.Structure):
    _fields_ = [("sht", ctypes.c_void_p), ("nfl", ctypes.c_int), ("spec_in", ctypes.c_void_p),
                ("grid", ctypes.c_void_p), ("spec_out", ctypes.c_void_p), ("ens", ctypes.c_void_p),
                ("ens_spec_in", ctypes.c_void_p), ("ens_grid", ctypes.c_void_p),
                ("ens_spec_out", ctypes.c_void_p), ("ens_nfl", ctypes.c_void_p),
                ("nremap", ctypes.c_int), ("remaps", ctypes.c_void_p), ("flux", ctypes.c_void_p),
                ("flux_grid", ctypes.c_void_p), ("implcpl", ctypes.c_void_p), ("implcpl_fwd", ctypes.c_void_p),
                ("nremap_post", ctypes.c_int), ("remaps_post", ctypes.c_void_p)]


class HostCopy(ctypes.Structure):
    _fields_ = [("host", ctypes.c_void_p), ("dev", ctypes.c_void_p), ("bytes", ctypes.c_size_t)]


def exported_symbols():
    """Names the C ABI exports (the declarations of include/dccm_gb300.h)."""
    return sorted(_SIGS)


def load(path=None):
    """Load the library (raises if it is missing: there is no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise ImportError("libdccm_gb300.so not built (%s); run __graft_entry__.build()" % path)
    L = ctypes.CDLL(path)
    for name, (res, args) in _SIGS.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def _check(st, what):
    if st != 0:
        raise DccmError(st, what)


def _p(a):
    """Pointer of a numpy array or a torch tensor (device or host)."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return ctypes.c_void_p(a.data_ptr())
    return a.ctypes.data_as(ctypes.c_void_p)


def _stream(s):
    if s is None:
        return None
    if hasattr(s, "cuda_stream"):
        return ctypes.c_void_p(s.cuda_stream)
    return ctypes.c_void_p(int(s))


def fp64_peak(stream=None):
    """dccm_fp64_peak: measured FP64 FMA throughput of the device, TFLOP/s."""
    v = ctypes.c_double()
    _check(load().dccm_fp64_peak(_stream(stream), ctypes.byref(v)), "dccm_fp64_peak")
    return v.value


FP64_RCP, FP64_EXP, FP64_LOG, FP64_SQRT, FP64_RSQRT = 0, 1, 2, 3, 4


def fp64_fn_dev(fn, x, y, stream=None):
    """dccm_fp64_fn_dev: the bulk-flux kernel's FP64 reciprocal (0), exp (1),
    log (2), square root (3) or reciprocal square root (4) of the float64
    device tensor x into y (same length), stream-ordered."""
    if x.numel() != y.numel():
        raise ValueError("x and y differ in length")
    _check(load().dccm_fp64_fn_dev(int(fn), ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()),
                                   int(x.numel()), _stream(stream)), "dccm_fp64_fn_dev")


def tune_set(knob, value):
    """dccm_tune_set: process-wide knob (launch shapes tc_shape, tc_ctas,
    fft_bb, fft_rpw, flux_threads, flux_ctas, remap_threads, remap_fc,
    serial, prio; host copies upload_order,
    host_path; failure path wait_limit_ms, tc_withhold_loads); 0 = the
    default."""
    _check(load().dccm_tune_set(knob.encode(), int(value)), "dccm_tune_set")


def tune_get(knob):
    v = ctypes.c_int()
    _check(load().dccm_tune_get(knob.encode(), ctypes.byref(v)), "dccm_tune_get")
    return v.value


# ------------------------------------------------------------- bulk flux
def DSFCM_Util_SfcBulkFlux_Get(arrays, IA, JA, IS, IE, JS, JE, device=False, stream=None):
    """Run the bulk flux on a dict of Fortran-ordered arrays (names of the
    reference's dummy arguments without the xy_/xya_/a_ prefixes, except
    a_Sig1Info).  Host numpy arrays use the host entry point; torch CUDA
    tensors with device=True use the device entry point."""
    L = load()
    a = FluxArgs()
    keep = []
    for n in FLUX_ARGS:
        arr = arrays[n]
        if n == "a_Sig1Info" and device:
            arr = np.ascontiguousarray(np.asarray(arr.cpu() if hasattr(arr, "cpu") else arr, np.float64))
            keep.append(arr)
        setattr(a, n, _p(arr).value)
    g = SfcGrid(IA, JA, IS, IE, JS, JE)
    if device:
        _check(L.dccm_sfc_bulk_flux_get_dev(ctypes.byref(a), ctypes.byref(g), _stream(stream)),
               "dccm_sfc_bulk_flux_get_dev")
    else:
        _check(L.dccm_sfc_bulk_flux_get(ctypes.byref(a), ctypes.byref(g)), "dccm_sfc_bulk_flux_get")


# ------------------------------------------------------------- remap table
class RemapTable:
    """Rows (iD, jD, iS, jS, w) of a Jones-99 table held by the library."""

    def __init__(self, handle):
        self.h = handle

    @property
    def nrow(self):
        n = ctypes.c_int64(0)
        _check(load().dccm_remap_table_size(self.h, ctypes.byref(n)), "dccm_remap_table_size")
        return n.value

    def rows(self):
        n = self.nrow
        bufs = [np.zeros(n, np.int32) for _ in range(4)] + [np.zeros(n, np.float64)]
        _check(load().dccm_remap_table_rows(self.h, *[_p(b) for b in bufs]), "dccm_remap_table_rows")
        return tuple(bufs)

    def write(self, path):
        _check(load().dccm_remap_table_write(self.h, path.encode()), "dccm_remap_table_write")

    def index(self, GNXS, GNXR):
        """set_mappingTable_interpCoef: (send_index, recv_index, coef), 1-based."""
        n = self.nrow
        s = np.zeros(n, np.int32)
        r = np.zeros(n, np.int32)
        c = np.zeros(n, np.float64)
        _check(load().dccm_remap_table_index(self.h, GNXS, GNXR, _p(s), _p(r), _p(c)), "dccm_remap_table_index")
        return s, r, c

    def __del__(self):
        if self.h and _lib is not None:
            _lib.dccm_remap_table_destroy(self.h)
            self.h = None


def gen_gridmapfile_lonlat2lonlat(x_LonS, y_LatS, x_LonD, y_LatD, x_LonIntWtS, y_LatIntWtS,
                                  x_LonIntWtD, y_LatIntWtD, accuracy_order=1, weight_mode=J99_REF,
                                  dst_mask=None):
    """Jones-99 table on the GPU (grid_mapping_util_jones99.f90:35-41)."""
    L = load()
    arrs = [np.ascontiguousarray(x, np.float64) for x in
            (x_LonS, y_LatS, x_LonD, y_LatD, x_LonIntWtS, y_LatIntWtS, x_LonIntWtD, y_LatIntWtD)]
    m = None if dst_mask is None else np.ascontiguousarray(dst_mask, np.uint8)
    h = ctypes.c_void_p()
    _check(L.dccm_j99_generate(_p(arrs[0]), len(arrs[0]), _p(arrs[1]), len(arrs[1]),
                               _p(arrs[2]), len(arrs[2]), _p(arrs[3]), len(arrs[3]),
                               _p(arrs[4]), _p(arrs[5]), _p(arrs[6]), _p(arrs[7]),
                               accuracy_order, weight_mode, _p(m), ctypes.byref(h)), "dccm_j99_generate")
    return RemapTable(h)


def bilinear_generate(x_LonS, y_LatS, x_LonR, y_LatR, dst_mask=None):
    """Bilinear table on the GPU (common/grid_mapping_util.f90:32-182)."""
    L = load()
    a = [np.ascontiguousarray(x, np.float64) for x in (x_LonS, y_LatS, x_LonR, y_LatR)]
    m = None if dst_mask is None else np.ascontiguousarray(dst_mask, np.uint8)
    h = ctypes.c_void_p()
    _check(L.dccm_bilinear_generate(_p(a[0]), len(a[0]), _p(a[1]), len(a[1]), _p(a[2]), len(a[2]),
                                    _p(a[3]), len(a[3]), _p(m), ctypes.byref(h)), "dccm_bilinear_generate")
    return RemapTable(h)


def exchange_grid(y_LatA, y_IntWtLatA, y_LatO, y_IntWtLatO):
    """Latitudes and sin-latitude widths of the surface exchange grid
    (tool/gmapgen/gmapgen_main.f90:336-405); longitudes are the atmosphere's."""
    a = [np.ascontiguousarray(x, np.float64) for x in (y_LatA, y_IntWtLatA, y_LatO, y_IntWtLatO)]
    n = len(a[0]) + len(a[2])
    lat, w = np.zeros(n), np.zeros(n)
    m = ctypes.c_int(0)
    _check(load().dccm_exchange_grid(_p(a[0]), _p(a[1]), len(a[0]), _p(a[2]), _p(a[3]), len(a[2]), _p(lat),
                                     _p(w), ctypes.byref(m)), "dccm_exchange_grid")
    return lat[:m.value], w[:m.value]


def gmapgen(A, O, conservative=True, orders=(1, 1, 1, 1, 1, 1), weight_mode=J99_REF):
    """The six tables of tool/gmapgen/gmapgen_main.f90:100-148 between the
    atmosphere grid A, the ocean grid O and their surface exchange grid S,
    each grid given as (x_Lon, y_Lat, x_IntWtLon, y_IntWtLat).  Returns
    (S, {"AO": table, "OA": ..., "AS", "SA", "OS", "SO"})."""
    latS, wS = exchange_grid(A[1], A[3], O[1], O[3])
    S = (np.asarray(A[0], np.float64), latS, np.asarray(A[2], np.float64), wS)
    grids = {"A": A, "O": O, "S": S}
    out = {}
    for k, tag in enumerate(("AO", "OA", "AS", "SA", "OS", "SO")):
        src, dst = grids[tag[0]], grids[tag[1]]
        if conservative:
            out[tag] = gen_gridmapfile_lonlat2lonlat(src[0], src[1], dst[0], dst[1], src[2], src[3], dst[2],
                                                     dst[3], accuracy_order=orders[k], weight_mode=weight_mode)
        else:
            out[tag] = bilinear_generate(src[0], src[1], dst[0], dst[1])
    return S, out


def read_table(path):
    h = ctypes.c_void_p()
    _check(load().dccm_remap_table_read(path.encode(), ctypes.byref(h)), "dccm_remap_table_read")
    return RemapTable(h)


def set_mappingTable_interpCoef(gridmapfile, GNXS, GNXR):
    """Reader of the reference text format (:446-506): (send_index, recv_index, coef)."""
    return read_table(gridmapfile).index(GNXS, GNXR)


# ------------------------------------------------------------- remap apply
class RemapPlan:
    """Operation list of one (recv, send, mapping_tag) triple on the device."""

    def __init__(self, n_send_points, n_recv_points, send_index, recv_index, coef):
        L = load()
        si = np.ascontiguousarray(send_index, np.int32)
        ri = np.ascontiguousarray(recv_index, np.int32)
        cf = np.ascontiguousarray(coef, np.float64)
        self.h = ctypes.c_void_p()
        self.n_send, self.n_recv = int(n_send_points), int(n_recv_points)
        _check(L.dccm_remap_plan_create(self.n_send, self.n_recv, len(si), _p(si), _p(ri), _p(cf),
                                        ctypes.byref(self.h)), "dccm_remap_plan_create")

    def info(self):
        a, b, c = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        _check(load().dccm_remap_plan_info(self.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)),
               "dccm_remap_plan_info")
        return a.value, b.value, c.value

    def interpolate_data(self, send_data, recv_data, num_of_data):
        """interpolate_data (interpolate_data.f90:1-15) on host arrays
        send_data(sn1,sn2), recv_data(rn1,rn2), Fortran order (modified in place)."""
        assert send_data.flags.f_contiguous and recv_data.flags.f_contiguous
        sn1, sn2 = send_data.shape
        rn1, rn2 = recv_data.shape
        _check(load().dccm_interpolate_data(self.h, sn1, sn2, _p(send_data), rn1, rn2, _p(recv_data),
                                            int(num_of_data)), "dccm_interpolate_data")

    def apply_dev(self, src, ld_src, dst, ld_dst, nfields, stream=None):
        _check(load().dccm_remap_apply_dev(self.h, _p(src), ld_src, _p(dst), ld_dst, nfields,
                                           _stream(stream)), "dccm_remap_apply_dev")

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.dccm_remap_plan_destroy(self.h)
            self.h = None


def area_integral_dev(f, area, stream=None):
    out = ctypes.c_double(0.0)
    _check(load().dccm_area_integral_dev(_p(f), _p(area), f.numel(), ctypes.byref(out), _stream(stream)),
           "dccm_area_integral_dev")
    return out.value


# ---------------------------------------------------- spectral operators
SPEC_LAPLACIAN, SPEC_INV_LAPLACIAN, SPEC_HDIFF_TENDENCY, SPEC_HDIFF_IMPLICIT = 0, 1, 2, 3


class SpecOp(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("radius", ctypes.c_double), ("order", ctypes.c_int),
                ("efold_time", ctypes.c_double), ("dt", ctypes.c_double), ("rotation_correction", ctypes.c_int)]


def spec_op(kind, radius, order=8, efold_time=1.0, dt=0.0, rotation_correction=False):
    """A dccm_spec_op: Laplacian, inverse Laplacian, hyperdiffusion tendency
    or implicit step (HDOrder = order, e-folding time of wavenumber nmax)."""
    return SpecOp(kind, radius, order, efold_time, dt, int(bool(rotation_correction)))


def spec_apply(nmax, op, spec):
    """dccm_spec_apply on host spectra complex128 [batch, ncoef]."""
    spec = np.ascontiguousarray(spec, np.complex128)
    out = np.empty_like(spec)
    _check(load().dccm_spec_apply(int(nmax), ctypes.byref(op), _p(spec), _p(out), spec.shape[0]),
           "dccm_spec_apply")
    return out


def spec_apply_dev(nmax, op, spec_in, spec_out, batch, stream=None):
    """dccm_spec_apply_dev on device spectra (float64 views of complex)."""
    _check(load().dccm_spec_apply_dev(int(nmax), ctypes.byref(op), _p(spec_in), _p(spec_out), int(batch),
                                      _stream(stream)), "dccm_spec_apply_dev")


# ------------------------------------------------------------------- SHT
class ShtPlan:
    """w_Initial(nMax, iMax, jMax) equivalent: a transform plan on the GPU.

    precision SHT_FP64 (CUDA cores) or SHT_MIXED (tcgen05 BF16x3 Legendre,
    FP32 FFT).  Spectra are complex128 [batch, ncoef] (m-major), grids
    float64 [batch, jmax, imax]."""

    def __init__(self, nmax, imax, jmax, precision=SHT_FP64, max_batch=1):
        L = load()
        self.N, self.I, self.J = int(nmax), int(imax), int(jmax)
        self.ncoef = (self.N + 1) * (self.N + 2) // 2
        self.precision = precision
        self.max_batch = int(max_batch)
        self.h = ctypes.c_void_p()
        _check(L.dccm_sht_plan_create(self.N, self.I, self.J, precision, self.max_batch, ctypes.byref(self.h)),
               "dccm_sht_plan_create")

    def axes(self):
        """(x_Lon, y_Lat, x_Lon_Weight, y_Lat_Weight) as SPML returns them."""
        a = [np.zeros(self.I), np.zeros(self.J), np.zeros(self.I), np.zeros(self.J)]
        _check(load().dccm_sht_axes(self.h, *[_p(x) for x in a]), "dccm_sht_axes")
        return tuple(a)

    def gauss(self):
        mu, w = np.zeros(self.J), np.zeros(self.J)
        _check(load().dccm_sht_gauss(self.h, _p(mu), _p(w)), "dccm_sht_gauss")
        return mu, w

    def pnm(self):
        p = np.zeros(self.ncoef * (self.J // 2))
        _check(load().dccm_sht_pnm(self.h, _p(p)), "dccm_sht_pnm")
        return p.reshape(self.ncoef, self.J // 2)

    def inverse(self, spec):
        spec = np.ascontiguousarray(spec, np.complex128)
        B = spec.shape[0]
        grid = np.zeros((B, self.J, self.I))
        _check(load().dccm_sht_inverse(self.h, _p(spec), _p(grid), B), "dccm_sht_inverse")
        return grid

    def forward(self, grid):
        grid = np.ascontiguousarray(grid, np.float64)
        B = grid.shape[0]
        spec = np.zeros((B, self.ncoef), np.complex128)
        _check(load().dccm_sht_forward(self.h, _p(grid), _p(spec), B), "dccm_sht_forward")
        return spec

    def inverse_dev(self, spec, grid, batch, stream=None):
        _check(load().dccm_sht_inverse_dev(self.h, _p(spec), _p(grid), int(batch), _stream(stream)),
               "dccm_sht_inverse_dev")

    def forward_dev(self, grid, spec, batch, stream=None):
        _check(load().dccm_sht_forward_dev(self.h, _p(grid), _p(spec), int(batch), _stream(stream)),
               "dccm_sht_forward_dev")

    def status(self):
        e = ctypes.c_int(0)
        st = load().dccm_sht_status(self.h, ctypes.byref(e))
        return st, e.value

    # SPML's real layout wa[b][l], l = l_nm(n, m) - 1 (see l_nm below)
    @property
    def nwa(self):
        return (self.N + 1) ** 2

    def xya_wa(self, wa):
        """SPML xya_wa: wa [batch, (N+1)^2] -> grid [batch, J, I] (host arrays)."""
        wa = np.ascontiguousarray(wa, np.float64)
        B = wa.shape[0]
        xya = np.zeros((B, self.J, self.I))
        _check(load().dccm_sht_xya_wa(self.h, _p(wa), _p(xya), B), "dccm_sht_xya_wa")
        return xya

    def wa_xya(self, xya):
        """SPML wa_xya: grid [batch, J, I] -> wa [batch, (N+1)^2] (host arrays)."""
        xya = np.ascontiguousarray(xya, np.float64)
        B = xya.shape[0]
        wa = np.zeros((B, self.nwa))
        _check(load().dccm_sht_wa_xya(self.h, _p(xya), _p(wa), B), "dccm_sht_wa_xya")
        return wa

    def xya_wa_dev(self, wa, xya, batch, stream=None):
        _check(load().dccm_sht_xya_wa_dev(self.h, _p(wa), _p(xya), int(batch), _stream(stream)),
               "dccm_sht_xya_wa_dev")

    def wa_xya_dev(self, xya, wa, batch, stream=None):
        _check(load().dccm_sht_wa_xya_dev(self.h, _p(xya), _p(wa), int(batch), _stream(stream)),
               "dccm_sht_wa_xya_dev")

    def spec_from_wa_dev(self, wa, spec, batch, stream=None):
        _check(load().dccm_sht_spec_from_wa_dev(self.h, _p(wa), _p(spec), int(batch), _stream(stream)),
               "dccm_sht_spec_from_wa_dev")

    def wa_from_spec_dev(self, spec, wa, batch, stream=None):
        _check(load().dccm_sht_wa_from_spec_dev(self.h, _p(spec), _p(wa), int(batch), _stream(stream)),
               "dccm_sht_wa_from_spec_dev")

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.dccm_sht_plan_destroy(self.h)
            self.h = None


def l_nm(n, m):
    """SPML's l_nm: 1-based position of total wavenumber n, zonal
    wavenumber m (-n <= m <= n) in a wa array: n(n+1) + m + 1; Re s_n^m at
    m >= 0, Im s_n^|m| at m < 0 (works element-wise on numpy arrays)."""
    return n * (n + 1) + m + 1


def nm_l(l):
    """SPML's nm_l: (n, m) of the 1-based wa position l (element-wise)."""
    l0 = np.asarray(l) - 1
    n = np.floor(np.sqrt(l0)).astype(np.int64)
    n = np.where((n + 1) ** 2 <= l0, n + 1, n)
    n = np.where(n * n > l0, n - 1, n)
    return n, l0 - n * (n + 1)


class Ensemble:
    """Truncation groups of an ensemble (dccm_sht_ensemble_create): one
    persistent Legendre launch and one FFT launch per direction on the
    mixed path.  groups: list of (nmax, imax, jmax, max_batch)."""

    def __init__(self, groups, precision=SHT_MIXED):
        L = load()
        ng = len(groups)
        arr = [(ctypes.c_int * ng)(*[int(g[k]) for g in groups]) for k in range(4)]
        self.groups = list(groups)
        self.h = ctypes.c_void_p()
        _check(L.dccm_sht_ensemble_create(ng, *arr, precision, ctypes.byref(self.h)), "dccm_sht_ensemble_create")

    def _call(self, fn, a, b, batch, stream):
        ng = len(self.groups)
        pa = (ctypes.c_void_p * ng)(*[_p(x).value for x in a])
        pb = (ctypes.c_void_p * ng)(*[_p(x).value for x in b])
        nb = (ctypes.c_int * ng)(*[int(x) for x in batch])
        _check(fn(self.h, pa, pb, nb, _stream(stream)), fn.__name__)

    def inverse_dev(self, spec, grid, batch, stream=None):
        self._call(load().dccm_sht_ensemble_inverse_dev, spec, grid, batch, stream)

    def forward_dev(self, grid, spec, batch, stream=None):
        self._call(load().dccm_sht_ensemble_forward_dev, grid, spec, batch, stream)

    def status(self):
        e = ctypes.c_int(0)
        st = load().dccm_sht_ensemble_status(self.h, ctypes.byref(e))
        return st, e.value

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.dccm_sht_ensemble_destroy(self.h)
            self.h = None


# ----------------------------------------------------------- coupling step
class HostCopies:
    """The copy lists of Step.run_host as the C arrays it passes: (host
    tensor or array, device tensor) pairs for the uploads and the
    downloads.  The buffers are kept referenced; they must stay allocated
    (and page-locked, if they were) while the lists are in use."""

    def __init__(self, h2d, d2h):
        self.pairs = (list(h2d), list(d2h))
        self.h2d, self.nh2d = self._array(self.pairs[0])
        self.d2h, self.nd2h = self._array(self.pairs[1])

    @staticmethod
    def _array(pairs):
        arr = (HostCopy * max(1, len(pairs)))()
        for k, (h, dv) in enumerate(pairs):
            nb = h.numel() * h.element_size() if hasattr(h, "numel") else h.nbytes
            arr[k] = HostCopy(_p(h).value, _p(dv).value, nb)
        return arr, len(pairs)

    def nbytes(self):
        """(bytes uploaded, bytes downloaded) per call."""
        return tuple(sum(c.bytes for c in arr[:n]) for arr, n in ((self.h2d, self.nh2d), (self.d2h, self.nd2h)))


class Step:
    """One coupling step as a CUDA graph (dccm_step_create).  Buffers are
    device tensors that must outlive the step; flux is a dict of device
    tensors keyed like DSFCM_Util_SfcBulkFlux_Get's arguments."""

    def __init__(self, sht=None, nfl=0, spec_in=None, grid=None, spec_out=None, remaps=(), flux=None,
                 flux_grid=None, ensemble=None, ens_spec_in=None, ens_grid=None, ens_spec_out=None, ens_nfl=None,
                 implcpl=None, implcpl_prof=None, implcpl_out=None, remaps_post=()):
        """remaps, remaps_post: sequences of (RemapPlan, nfields, src, ld_src,
        dst, ld_dst[, nsub, ld_dst2]).  implcpl: an ImplCplPlan whose forward
        sweep (profiles implcpl_prof, outputs implcpl_out: dicts of device
        tensors as ImplCplPlan.forward_dev takes) runs before the remaps and
        whose backward sweep runs after the flux and remaps_post."""
        L = load()
        d = StepDesc()
        d.sht = sht.h.value if sht is not None else None
        d.nfl = int(nfl)
        d.spec_in, d.grid, d.spec_out = (_p(x).value if x is not None else None for x in (spec_in, grid, spec_out))
        self._keep = [sht, spec_in, grid, spec_out, flux, remaps, ensemble, ens_spec_in, ens_grid, ens_spec_out]
        if ensemble is not None:
            ng = len(ens_nfl)
            self._ens = [(ctypes.c_void_p * ng)(*[_p(x).value for x in arrs])
                         for arrs in (ens_spec_in, ens_grid, ens_spec_out)]
            self._ens_nfl = (ctypes.c_int * ng)(*[int(x) for x in ens_nfl])
            d.ens = ensemble.h.value
            d.ens_spec_in, d.ens_grid, d.ens_spec_out = (ctypes.addressof(a) for a in self._ens)
            d.ens_nfl = ctypes.addressof(self._ens_nfl)
        def remap_array(lst):
            arr = (StepRemap * max(1, len(lst)))()
            for k, rm in enumerate(lst):
                plan, nf, src, lds, dst, ldd = rm[:6]
                nsub, ld2 = (rm[6], rm[7]) if len(rm) > 6 else (0, 0)
                arr[k] = StepRemap(plan.h.value, int(nf), _p(src).value, int(lds), _p(dst).value, int(ldd),
                                   int(nsub), int(ld2))
            return arr
        self._remaps = remap_array(remaps)
        d.nremap = len(remaps)
        d.remaps = ctypes.addressof(self._remaps)
        self._remaps_post = remap_array(remaps_post)
        d.nremap_post = len(remaps_post)
        d.remaps_post = ctypes.addressof(self._remaps_post)
        if implcpl is not None:
            self._icf = implcpl._args(implcpl_prof, implcpl_out)
            d.implcpl = implcpl.h.value
            d.implcpl_fwd = ctypes.addressof(self._icf)
            self._keep += [implcpl, implcpl_prof, implcpl_out, remaps_post]
        if flux is not None:
            fa = FluxArgs()
            self._sig = np.ascontiguousarray(np.asarray(flux["a_Sig1Info"], np.float64))
            for n in FLUX_ARGS:
                setattr(fa, n, self._sig.ctypes.data if n == "a_Sig1Info" else _p(flux[n]).value)
            self._fa = fa
            self._fg = SfcGrid(*flux_grid)
            d.flux = ctypes.addressof(fa)
            d.flux_grid = ctypes.addressof(self._fg)
        self.h = ctypes.c_void_p()
        _check(L.dccm_step_create(ctypes.byref(d), ctypes.byref(self.h)), "dccm_step_create")

    def run(self, stream=None):
        _check(load().dccm_step_run(self.h, _stream(stream)), "dccm_step_run")

    STAGES = ["legendre_inverse", "fft_inverse", "fft_forward", "legendre_forward", "remap", "bulk_flux"]
    KNOBS = ["tc_ctas", "fft_bb", "flux_threads", "remap_threads"]

    def autotune(self, cache_path=None):
        """dccm_step_autotune: choose launch shapes, re-record the graph."""
        out = (ctypes.c_int * 4)()
        _check(load().dccm_step_autotune(self.h, cache_path.encode() if cache_path else None, out),
               "dccm_step_autotune")
        chosen = dict(zip(self.KNOBS, list(out)))
        chosen["serial"] = tune_get("serial")
        chosen["flux_ctas"] = tune_get("flux_ctas")
        chosen["remap_fc"] = tune_get("remap_fc")
        chosen["tc_shape"] = tune_get("tc_shape")
        chosen["fft_rpw"] = tune_get("fft_rpw")
        chosen["prio"] = tune_get("prio")
        return chosen

    def run_timed(self, stream=None):
        """Device ms of the six stages (names in Step.STAGES), run back to back."""
        ms = (ctypes.c_float * 6)()
        _check(load().dccm_step_run_timed(self.h, _stream(stream), ms), "dccm_step_run_timed")
        return list(ms)

    def run_host(self, h2d, d2h=None, stream=None):
        """dccm_step_run_host.  h2d / d2h: lists of (host tensor or array,
        device tensor) pairs, or h2d a HostCopies holding both lists (built
        once, for a caller that passes the same buffers every step)."""
        c = h2d if isinstance(h2d, HostCopies) else HostCopies(h2d, d2h or [])
        _check(load().dccm_step_run_host(self.h, _stream(stream), c.h2d, c.nh2d, c.d2h, c.nd2h),
               "dccm_step_run_host")

    def launch_host(self, h2d, d2h=None, stream=None):
        """dccm_step_launch_host: run_host without the final synchronisation
        (page-locked buffers only); the downloads are in host memory once
        the stream has synchronised."""
        c = h2d if isinstance(h2d, HostCopies) else HostCopies(h2d, d2h or [])
        _check(load().dccm_step_launch_host(self.h, _stream(stream), c.h2d, c.nh2d, c.d2h, c.nd2h),
               "dccm_step_launch_host")

    def autotune_host(self, h2d, d2h=None, stream=None):
        """dccm_step_autotune_host: upload order, copy path and flux CTA cap
        for these copy lists, by timing (the step runs about 420 times);
        host_path is 1 + the mask of copy groups moved through the host
        mapping (bit 4: the flux kernel reads and writes its host rows
        itself), flux_ctas 0 the flux kernel's full grid."""
        c = h2d if isinstance(h2d, HostCopies) else HostCopies(h2d, d2h or [])
        out = (ctypes.c_int * 3)()
        ms = (ctypes.c_float * 32)()
        _check(load().dccm_step_autotune_host(self.h, _stream(stream), c.h2d, c.nh2d, c.d2h, c.nd2h, out, ms),
               "dccm_step_autotune_host")
        return {"upload_order": out[0], "host_path": out[1], "flux_ctas": out[2],
                "candidates_ms": {"%d,%d" % (1 + k // 16, 1 + k % 16): ms[k] for k in range(32)}}

    def host_choice(self, upload_order=0, host_path=0, flux_ctas=-1):
        """dccm_step_host_choice: this step's upload order, copy path and
        host-graph flux CTA cap (0, 0, -1: the process-wide knobs)."""
        _check(load().dccm_step_host_choice(self.h, int(upload_order), int(host_path), int(flux_ctas)),
               "dccm_step_host_choice")

    def host_release(self):
        """dccm_step_host_release: forget the recorded copy graph."""
        _check(load().dccm_step_host_release(self.h), "dccm_step_host_release")

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.dccm_step_destroy(self.h)
            self.h = None


# ------------------------------------------------------- implicit coupling
class ImplCplPlan:
    """SfcImplicitCoupling_VDiffForward / _VDiffBackward
    (atm/dcpam_sfc_implicit_coupling_mod.f90:72-378, :25-70) over ncol
    columns of kmax levels; the plan keeps the eliminated matrices (the
    reference's module state) between the two sweeps.  Arrays are the
    reference's with the columns flattened, given row-major as [k][c]
    (tracers [n][k][c], coefficients [a][c]); numpy arrays for the host
    entry points, CUDA tensors for the device ones."""

    def __init__(self, ncol, kmax, ncmax=1, index_h2ovap=1, consts=(9.8, 1004.6, 287.04, 1200.0)):
        self.ncol, self.kmax, self.ncmax = int(ncol), int(kmax), int(ncmax)
        self.consts = ImplCplConsts(*[float(x) for x in consts])
        h = ctypes.c_void_p()
        _check(load().dccm_implcpl_create(self.ncol, self.kmax, self.ncmax, int(index_h2ovap),
                                          ctypes.byref(self.consts), ctypes.byref(h)), "dccm_implcpl_create")
        self.h = h

    def _args(self, prof, out):
        a = ImplCplForwardArgs()
        names = {"xyr_MomFluxX": "MomFluxX", "xyr_MomFluxY": "MomFluxY", "xyr_HeatFlux": "HeatFlux",
                 "xyrf_QMixFlux": "QMixFlux", "xyr_Press": "Press", "xyz_Exner": "ExnerFull",
                 "xyr_Exner": "ExnerHalf", "xyr_VirTemp": "VirTemp", "xyz_Height": "Height",
                 "xyr_VelDiffCoef": "VelDiffCoef", "xyr_TempDiffCoef": "TempDiffCoef",
                 "xyr_QMixDiffCoef": "QMixDiffCoef", "xyz_DUDt": "DUDt", "xyz_DVDt": "DVDt",
                 "xyz_DTempDt": "DTempDt", "xyzf_DQMixDt": "DQMixDt", "xya_ImplCplCoef1": "ImplCplCoef1",
                 "xya_ImplCplCoef2": "ImplCplCoef2"}
        for f, n in names.items():
            x = prof.get(n) if n in prof else out[n]
            setattr(a, f, _p(x).value)
        return a

    def forward(self, prof):
        """Host arrays in (synth.column_profiles layout); returns the
        tendencies and coupling coefficients as numpy arrays."""
        K, n, nc = self.kmax, self.ncol, self.ncmax
        prof = {k: np.ascontiguousarray(v, dtype=np.float64) for k, v in prof.items()}
        out = {"DUDt": np.empty((K, n)), "DVDt": np.empty((K, n)), "DTempDt": np.empty((K, n)),
               "DQMixDt": np.empty((nc, K, n)), "ImplCplCoef1": np.empty((4, n)), "ImplCplCoef2": np.empty((4, n))}
        a = self._args(prof, out)
        _check(load().dccm_implcpl_forward(self.h, ctypes.byref(a)), "dccm_implcpl_forward")
        return out

    def forward_dev(self, prof, out, stream=None):
        """Device tensors in and out (same shapes as forward); stream-ordered."""
        a = self._args(prof, out)
        _check(load().dccm_implcpl_forward_dev(self.h, ctypes.byref(a), _stream(stream)), "dccm_implcpl_forward_dev")

    def backward(self, tend):
        """Host arrays DUDt, DVDt, DTempDt, DQMixDt, updated in place."""
        for k in ("DUDt", "DVDt", "DTempDt", "DQMixDt"):
            assert tend[k].dtype == np.float64 and tend[k].flags.c_contiguous
        _check(load().dccm_implcpl_backward(self.h, *[_p(tend[k]) for k in ("DUDt", "DVDt", "DTempDt", "DQMixDt")]),
               "dccm_implcpl_backward")

    def backward_dev(self, tend, stream=None):
        _check(load().dccm_implcpl_backward_dev(self.h, *[_p(tend[k]) for k in ("DUDt", "DVDt", "DTempDt", "DQMixDt")],
                                                _stream(stream)), "dccm_implcpl_backward_dev")

    def info(self):
        """dccm_implcpl_info: (ncol, kmax, ncmax)."""
        v = [ctypes.c_int() for _ in range(3)]
        _check(load().dccm_implcpl_info(self.h, *[ctypes.byref(x) for x in v]), "dccm_implcpl_info")
        return tuple(x.value for x in v)

    def matrices(self):
        """The module-state matrices (UVMtx, TempMtx, QMixMtx), each [3][kmax][ncol]."""
        m = {k: np.empty((3, self.kmax, self.ncol)) for k in ("UVMtx", "TempMtx", "QMixMtx")}
        _check(load().dccm_implcpl_matrices(self.h, _p(m["UVMtx"]), _p(m["TempMtx"]), _p(m["QMixMtx"])),
               "dccm_implcpl_matrices")
        return m

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.dccm_implcpl_destroy(self.h)
            self.h = None

