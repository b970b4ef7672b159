/*
 * CPU oracle for the Dennou-CCM coupling-step hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is what the CUDA library's
 * results are compared against, and the timed CPU baseline of bench.py.
 * No product code path loads it.
 *
 * It is a plain-C FP64 restatement of the reference algorithms:
 *   - surface bulk flux:  sfc/DSFCM_Util_SfcBulkFlux_mod.f90:35-58,108-591
 *   - Jones-99 table:     common/grid_mapping_util_jones99.f90:35-442
 *   - table reader:       common/grid_mapping_util_jones99.f90:446-506
 *   - remap apply:        common/interpolation_data_latlon_mod.f90:274-306
 *   - implicit coupling:  atm/dcpam_sfc_implicit_coupling_mod.f90:25-420
 *   - bilinear table:     common/grid_mapping_util.f90:32-182
 *   - exchange grid:      tool/gmapgen/gmapgen_main.f90:336-425
 *   - spherical-harmonic transform: SPML/ISPACK (external, not vendored);
 *     restated from the mathematics with the convention documented in
 *     oracle_sht.c.
 *
 * PARITY UNPINNED: the reference is Fortran 90 and no Fortran compiler,
 * nor its libraries (jcup, gtool5, SPML, ISPACK), exists where this is
 * built, and the reference ships no golden vectors or tests.  The oracle
 * is cross-checked instead against an independent numpy restatement
 * (tests/golden/make_golden.py), numpy's Gauss-Legendre nodes, and
 * analytic known answers.
 *
 * Compile with -ffp-contract=off so that results do not depend on whether
 * the host compiler fuses multiply-adds (GCC fuses by default on aarch64).
 */
#ifndef DCCM_ORACLE_H
#define DCCM_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- flux */
/* Pointer table in the dummy-argument order of DSFCM_Util_SfcBulkFlux_Get
 * (sfc/DSFCM_Util_SfcBulkFlux_mod.f90:108-120).  Index: */
enum {
  OF_WindStressX = 0, OF_WindStressY, OF_SenHFlx, OF_QVapMFlx, OF_LatHFlx,
  OF_SfcVelTransCoef, OF_SfcTempTransCoef, OF_SfcQVapTransCoef,
  OF_DelVarImplCPL, OF_SUwRFlx, OF_LUwRFlx, OF_SfcHFlx_ns, OF_SfcHFlx_sr,
  OF_DSfcHFlxDTs, OF_WindU, OF_WindV, OF_SfcAirTemp, OF_QVap1, OF_SDwRFlx,
  OF_LDwRFlx, OF_ImplCplCoef1, OF_ImplCplCoef2, OF_SfcTemp, OF_SfcAlbedo,
  OF_SIceCon, OF_Sig1Info, OF_SfcHeight, OF_SfcPress, OF_NARGS
};
/* Fortran bounds IS..IE, JS..JE (1-based) inside arrays of shape (IA,JA[,k]). */
void oracle_sfc_bulk_flux(double *const *args, int IA, int JA, int IS, int IE,
                          int JS, int JE);

/* --------------------------------------------------------------- remap */
/* Jones-99 table generation.  mode 0 = the reference's weights (REF),
 * mode 1 = true longitude overlap (conservative).  order 1 or 2.
 * Rows are (iD, jD, iS, jS, w) with 1-based grid indices exactly as the
 * reference writes them.  If cap is too small, *nrow is set to the needed
 * count and 1 is returned.  Returns <0 on a failed search (the reference
 * stops there). */
int oracle_j99_gen(const double *lonS, int nxs, const double *latS, int nys,
                   const double *lonD, int nxd, const double *latD, int nyd,
                   const double *latwtS, const double *latwtD, int order,
                   int mode, int64_t cap, int32_t *iD, int32_t *jD, int32_t *iS,
                   int32_t *jS, double *w, int64_t *nrow);

/* set_mappingTable_interpCoef: 1-based linear indices. */
void oracle_table_to_index(int64_t n, const int32_t *iD, const int32_t *jD,
                           const int32_t *iS, const int32_t *jS, int GNXS,
                           int GNXR, int32_t *send_index, int32_t *recv_index);

/* interpolate_data_latlon: recv(:,:)=0 then COO scatter-add in table order.
 * send is (sn1, num_of_data), recv is (rn1, num_of_data), column-major.
 * Returns -1 if an index is outside 1..sn1 or 1..rn1. */
int oracle_remap_apply(int64_t nop, const int32_t *send_index,
                       const int32_t *recv_index, const double *coef,
                       int64_t sn1, const double *send, int64_t rn1,
                       double *recv, int num_of_data);

/* Compensated (Neumaier) FP64 sum of f[i]*area[i]. */
double oracle_area_integral(int64_t n, const double *f, const double *area);

/* ----------------------------------------------------------------- SHT */
void oracle_gauss_nodes(int J, double *mu, double *w);
/* P-bar table, m-major: p[(idx(m,n))*J + j] for the J Gaussian nodes. */
void oracle_pnm(int N, int J, const double *mu, double *p);
/* Inverse: spec[b][ncoef] complex (re,im interleaved) -> grid[b][J][I]. */
void oracle_sht_inverse(int N, int I, int J, int batch, const double *spec,
                        double *grid);
/* Forward: grid[b][J][I] -> spec[b][ncoef] complex. */
void oracle_sht_forward(int N, int I, int J, int batch, const double *grid,
                        double *spec);
/* Real DFT of one row (FFT, any I = 2^a 3^b 5^c); out[m] m=0..M-1 complex,
 * out = (1/I) sum_i g_i e^{-2 pi i m i / I}. */
void oracle_rfft_row(int I, const double *g, int M, double *out);

void oracle_set_threads(int n);
int oracle_get_threads(void);

/* ------------------------------------------------------ implicit coupling */
/* SfcImplicitCoupling_VDiffForward (atm/dcpam_sfc_implicit_coupling_mod.f90:
 * 72-378) and VDiffBackward (:25-70) over ncol columns of kmax levels;
 * layouts in oracle_implcpl.c.  in[] / out[] indices: */
enum {
  OI_MomFluxX = 0, OI_MomFluxY, OI_HeatFlux, OI_QMixFlux, OI_Press, OI_ExnerFull,
  OI_ExnerHalf, OI_VirTemp, OI_Height, OI_VelDiffCoef, OI_TempDiffCoef,
  OI_QMixDiffCoef, OI_NIN
};
enum { OO_DUDt = 0, OO_DVDt, OO_DTempDt, OO_DQMixDt, OO_ImplCplCoef1, OO_ImplCplCoef2, OO_NOUT };
/* consts = {Grav, CpDry, GasRDry, DelTime}; ih2o is IndexH2OVap (1-based).
 * uv, tm, qm receive the eliminated matrices (ncol, kmax, -1:1). */
void oracle_implcpl_forward(const double *const *in, double *const *out, double *uv, double *tm,
                            double *qm, int64_t ncol, int kmax, int ncmax, int ih2o,
                            const double *consts);
void oracle_implcpl_backward(const double *uv, const double *tm, const double *qm, double *DUDt,
                             double *DVDt, double *DTempDt, double *DQMixDt, int64_t ncol, int kmax,
                             int ncmax, double DelTime);

/* ------------------------------------------- bilinear table, exchange grid */
/* gen_gridmapfile_lonlat2lonlat (common/grid_mapping_util.f90:32-182):
 * rows (iR, jR, iS, jS, w) in the reference's order.  Returns 1 (and the
 * needed *nrow) if cap is too small.  North of the last source latitude
 * (undefined in the reference) the rows extrapolate from the last two
 * source latitudes; -1 if there is only one. */
int oracle_bilin_gen(const double *lonS, int nxs, const double *latS, int nys, const double *lonR, int nxr,
                     const double *latR, int nyr, int64_t cap, int32_t *iR, int32_t *jR, int32_t *iS,
                     int32_t *jS, double *w, int64_t *nrow);
/* generate_surface_exchage_grid (tool/gmapgen/gmapgen_main.f90:336-405):
 * latitudes and sin-latitude widths of the surface exchange grid (its
 * longitudes are the atmosphere's).  latX, wX hold JMA + JMO entries;
 * returns JMS. */
int oracle_exchange_grid_lat(const double *latA, const double *wA, int JMA, const double *latO,
                             const double *wO, int JMO, double *latX, double *wX);

/* ------------------------------------------------ spectral-space operators */
/* Per-wavenumber scalings of [batch][ncoef] complex spectra (m-major):
 * kind 0 Laplacian, 1 inverse Laplacian, 2 hyperdiffusion tendency,
 * 3 implicit hyperdiffusion step; formulas in oracle_spec.c.  Returns -1
 * on invalid parameters.  in may equal out. */
int oracle_spec_apply(int N, int kind, double radius, int order, double efold_time, double dt,
                      int rotation_correction, int batch, const double *in, double *out);

#ifdef __cplusplus
}
#endif
#endif
