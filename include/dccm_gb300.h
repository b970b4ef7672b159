/*
 * dccm_gb300 — C ABI of the GB300 (sm_103a) implementation of the
 * Dennou-CCM per-coupling-step hot path:
 *   - surface bulk flux        (replaces sfc/DSFCM_Util_SfcBulkFlux_mod.f90)
 *   - Jones-99 remap table and its apply (replaces
 *     common/grid_mapping_util_jones99.f90 and
 *     common/interpolation_data_latlon_mod.f90 / interpolate_data.f90)
 *   - spherical-harmonic transform pair on the Gaussian grid (replaces the
 *     SPML w_module transforms that the atmosphere dynamics call)
 *   - the fused coupling step (all of the above, captured as a CUDA graph).
 *
 * Conventions shared by every entry point:
 *   - plain C types only; every function returns an int status
 *     (DCCM_OK = 0, negative on error; nothing aborts or throws);
 *   - arrays are Fortran column-major FP64 as in the reference;
 *   - "_dev" entry points take device pointers and a CUDA stream
 *     (passed as void*, NULL = default stream) and are stream-ordered;
 *     the others take host pointers and return when the results are in
 *     host memory (what a Fortran caller through iso_c_binding passes);
 *   - plans own their device memory and are not safe to use from two
 *     threads at once.
 */
#ifndef DCCM_GB300_H
#define DCCM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DCCM_ABI_VERSION 1

enum dccm_status {
  DCCM_OK = 0,
  DCCM_ERR_INVALID_ARG = -1,  /* null pointer, negative size, bad enum */
  DCCM_ERR_SHAPE = -2,        /* sizes inconsistent with the plan */
  DCCM_ERR_CUDA = -3,         /* a CUDA runtime call failed */
  DCCM_ERR_INDEX_RANGE = -4,  /* a table index outside the grid */
  DCCM_ERR_SEARCH = -5,       /* overlap search failed (the reference stops) */
  DCCM_ERR_IO = -6,           /* table file could not be read or written */
  DCCM_ERR_NOMEM = -7,        /* host or device allocation failed */
  DCCM_ERR_TIMEOUT = -8,      /* a bounded device wait gave up */
  DCCM_ERR_UNSUPPORTED = -9   /* size or mode the library does not handle */
};

/* Message for a status code (static storage). */
const char *dccm_status_string(int status);
/* DCCM_ABI_VERSION of the loaded library. */
int dccm_abi_version(void);
/* The last CUDA error code seen by the library on this thread (0 if none). */
int dccm_last_cuda_error(void);

/* =====================================================================
 * Surface bulk flux
 * Replaces DSFCM_Util_SfcBulkFlux_Get (sfc/DSFCM_Util_SfcBulkFlux_mod.f90:108-151)
 * and its module state IA, IS, IE, JA, JS, JE (sfc/DSFCM_Admin_Grid_mod.f90:35-52).
 * Members are in the Fortran dummy-argument order.  Arrays are (IA,JA),
 * (IA,JA,3) or (IA,JA,4) column-major; only the interior IS..IE x JS..JE
 * (1-based, inclusive) is read or written.  a_Sig1Info always points to
 * two host doubles.  Slot 3 of SfcHFlx_ns, SfcHFlx_sr and DSfcHFlxDTs is
 * left untouched, as in the reference.  Two reference behaviours are
 * given one defined meaning: the sea-ice flag of the final loop is taken
 * per surface type (the reference's OpenMP loop shares it between types,
 * :384-393), and slot 3 of LatHFlx after the implicit correction is the
 * fraction-weighted merge of slots 1 and 2 (the reference reads a
 * latent-heat array of extent 2 at index 3, :379).
 * ===================================================================== */
typedef struct dccm_sfc_bulk_flux_args {
  double *WindStressX, *WindStressY;                          /* out (IA,JA,3) */
  double *SenHFlx, *QVapMFlx, *LatHFlx;                       /* out (IA,JA,3) */
  double *SfcVelTransCoef, *SfcTempTransCoef, *SfcQVapTransCoef; /* out (IA,JA,3) */
  double *DelVarImplCPL;                                      /* out (IA,JA,4) */
  double *SUwRFlx, *LUwRFlx;                                  /* out (IA,JA,3) */
  double *SfcHFlx_ns, *SfcHFlx_sr, *DSfcHFlxDTs;              /* out (IA,JA,3), slot 3 untouched */
  const double *WindU, *WindV, *SfcAirTemp, *QVap1;           /* in (IA,JA) */
  const double *SDwRFlx, *LDwRFlx;                            /* in (IA,JA) */
  const double *ImplCplCoef1, *ImplCplCoef2;                  /* in (IA,JA,4) */
  double *SfcTemp, *SfcAlbedo;                                /* inout (IA,JA,3) */
  const double *SIceCon;                                      /* in (IA,JA) */
  const double *a_Sig1Info;                                   /* in, 2 host doubles */
  const double *SfcHeight, *SfcPress;                         /* in (IA,JA) */
} dccm_sfc_bulk_flux_args;

typedef struct dccm_sfc_grid {
  int IA, JA; /* array extents including halo */
  int IS, IE; /* interior, 1-based inclusive */
  int JS, JE;
} dccm_sfc_grid;

/* Host arrays; returns after the outputs are back in host memory. */
int dccm_sfc_bulk_flux_get(const dccm_sfc_bulk_flux_args *args,
                           const dccm_sfc_grid *grid);
/* Device arrays (a_Sig1Info stays a host pointer); stream-ordered. */
int dccm_sfc_bulk_flux_get_dev(const dccm_sfc_bulk_flux_args *args,
                               const dccm_sfc_grid *grid, void *stream);

/* =====================================================================
 * Implicit surface coupling of the atmosphere's vertical diffusion: the
 * producer of the bulk flux's ImplCplCoef1/2 and the consumer of its
 * DelVarImplCPL.
 * dccm_implcpl_forward[_dev] replaces SfcImplicitCoupling_VDiffForward
 * (atm/dcpam_sfc_implicit_coupling_mod.f90:72-378, with
 * Solve_TriDiagSystem_Forward :380-405); dccm_implcpl_backward[_dev]
 * replaces SfcImplicitCoupling_VDiffBackward (:25-70, with
 * Solve_TriDiagSystem_Backward :407-420).  The plan holds what the
 * reference keeps as module state (xyza_UVMtx, xyza_TempMtx,
 * xyza_QMixMtx, allocated by dcpam_sfc_implicit_coupling_Init :422-428)
 * from the forward sweep to the backward one.  Arrays are the reference's,
 * columns (i, j) flattened to ncol = imax*jmax: xyr_* (ncol, 0:kmax),
 * xyz_* (ncol, kmax), xyrf_QMixFlux (ncol, 0:kmax, ncmax), xyzf_DQMixDt
 * (ncol, kmax, ncmax), xya_ImplCplCoef1/2 (ncol, 4), column-major.
 * Level 1 of the forward sweep's tendencies divides by the zero
 * sub-diagonal the reference sets at k = 1 and holds its infinities or
 * NaN; the coupler replaces U, V, T and the vapour tracer there with the
 * surface solution (DelVarImplCPL) before the backward sweep
 * (atm/dccm_atm_mod.f90:832-835), as a caller must.  FP64; agrees with
 * the reference's operation order to rounding.
 * ===================================================================== */
typedef struct dccm_implcpl dccm_implcpl;
/* Constants of the `constants' and `timeset' modules the routines use. */
typedef struct dccm_implcpl_consts {
  double Grav, CpDry, GasRDry, DelTime;
} dccm_implcpl_consts;
typedef struct dccm_implcpl_forward_args {
  const double *xyr_MomFluxX, *xyr_MomFluxY, *xyr_HeatFlux; /* in (ncol, 0:kmax) */
  const double *xyrf_QMixFlux;                              /* in (ncol, 0:kmax, ncmax) */
  const double *xyr_Press, *xyz_Exner, *xyr_Exner;          /* in */
  const double *xyr_VirTemp, *xyz_Height;                   /* in */
  const double *xyr_VelDiffCoef, *xyr_TempDiffCoef, *xyr_QMixDiffCoef; /* in (ncol, 0:kmax) */
  double *xyz_DUDt, *xyz_DVDt, *xyz_DTempDt;                /* out (ncol, kmax) */
  double *xyzf_DQMixDt;                                     /* out (ncol, kmax, ncmax) */
  double *xya_ImplCplCoef1, *xya_ImplCplCoef2;              /* out (ncol, 4) */
} dccm_implcpl_forward_args;

/* index_h2ovap: IndexH2OVap, 1-based tracer of the vapour (1..ncmax); kmax >= 2. */
int dccm_implcpl_create(int ncol, int kmax, int ncmax, int index_h2ovap,
                        const dccm_implcpl_consts *consts, dccm_implcpl **plan);
int dccm_implcpl_destroy(dccm_implcpl *plan);
/* Host arrays; returns when the outputs are in host memory. */
int dccm_implcpl_forward(dccm_implcpl *plan, const dccm_implcpl_forward_args *args);
/* Device arrays; stream-ordered. */
int dccm_implcpl_forward_dev(dccm_implcpl *plan, const dccm_implcpl_forward_args *args,
                             void *stream);
/* In place on the tendencies (after level 1 has been replaced). */
int dccm_implcpl_backward(dccm_implcpl *plan, double *xyz_DUDt, double *xyz_DVDt,
                          double *xyz_DTempDt, double *xyzf_DQMixDt);
int dccm_implcpl_backward_dev(dccm_implcpl *plan, double *xyz_DUDt, double *xyz_DVDt,
                              double *xyz_DTempDt, double *xyzf_DQMixDt, void *stream);
/* Copies the module-state matrices out, each (ncol, kmax, -1:1); NULL skips one. */
int dccm_implcpl_matrices(dccm_implcpl *plan, double *uv, double *temp, double *qmix);
/* The plan's shape (any pointer may be NULL). */
int dccm_implcpl_info(const dccm_implcpl *plan, int *ncol, int *kmax, int *ncmax);

/* =====================================================================
 * Jones-99 remap table
 * dccm_j99_generate replaces gen_gridmapfile_lonlat2lonlat
 * (common/grid_mapping_util_jones99.f90:35-41, body :78-442); the table is
 * built on the GPU and returned in host memory instead of a text file.
 * Grid arguments are those of the reference: centre longitudes and
 * latitudes (radians, latitudes ascending south to north) and integration
 * weights (x_*IntWt* is accepted and unused, as in the reference; y_*IntWt*
 * are the sin-latitude widths, sum 2).
 *   weight_mode DCCM_J99_REF      the reference's weights and pattern,
 *                                 rows identical to the reference file;
 *   weight_mode DCCM_J99_CONSERVE true longitude overlaps: row sums 1 and
 *                                 global integrals conserved for any grids.
 * dst_mask (nxd*nyd bytes, i fastest, or NULL) drops rows of destination
 * cells whose mask is 0 (land); the reference's masks are all true.
 * accuracy_order 1 or 2 (second-order adds the latitude-gradient rows).
 * ===================================================================== */
enum { DCCM_J99_REF = 0, DCCM_J99_CONSERVE = 1 };

typedef struct dccm_remap_table dccm_remap_table;

int dccm_j99_generate(const double *x_LonS, int nxs, const double *y_LatS, int nys,
                      const double *x_LonD, int nxd, const double *y_LatD, int nyd,
                      const double *x_LonIntWtS, const double *y_LatIntWtS,
                      const double *x_LonIntWtD, const double *y_LatIntWtD,
                      int accuracy_order, int weight_mode, const uint8_t *dst_mask,
                      dccm_remap_table **table);
/* dccm_bilinear_generate replaces gen_gridmapfile_lonlat2lonlat of
 * common/grid_mapping_util.f90:32-182 (the bilinear mapping of the
 * coupler's non-conservative tags, tool/gmapgen/gmapgen_main.f90:100-117):
 * four rows per destination cell (two per source column, or one outside
 * the source latitudes, when either grid has a single longitude), in the
 * reference's order, weights bit-identical to the reference's.  North of
 * the last source latitude the reference reads past its latitude array;
 * there the rows extrapolate linearly from the last two source latitudes,
 * as the reference itself does south of the first.  Longitudes are assumed
 * uniform and starting at 0, as the reference's index formula does.
 * dst_mask as for dccm_j99_generate.  Returns DCCM_ERR_UNSUPPORTED for a
 * single source latitude on a grid that is not axisymmetric. */
int dccm_bilinear_generate(const double *x_LonS, int nxs, const double *y_LatS, int nys,
                           const double *x_LonR, int nxr, const double *y_LatR, int nyr,
                           const uint8_t *dst_mask, dccm_remap_table **table);
/* generate_surface_exchage_grid (tool/gmapgen/gmapgen_main.f90:336-405):
 * latitudes (radians) and sin-latitude widths of the surface exchange grid
 * from the atmosphere's and the ocean's; its longitudes are the
 * atmosphere's.  y_LatX and y_IntWtLatX hold JMA + JMO values; *JMX
 * receives the count.  Host arithmetic. */
int dccm_exchange_grid(const double *y_LatA, const double *y_IntWtLatA, int JMA,
                       const double *y_LatO, const double *y_IntWtLatO, int JMO,
                       double *y_LatX, double *y_IntWtLatX, int *JMX);
/* Number of rows (iD, jD, iS, jS, w). */
int dccm_remap_table_size(const dccm_remap_table *table, int64_t *nrow);
/* Copies the rows out (1-based grid indices as in the reference file). */
int dccm_remap_table_rows(const dccm_remap_table *table, int32_t *iD, int32_t *jD,
                          int32_t *iS, int32_t *jS, double *w);
/* Writes / reads the reference's text format: one "iD jD iS jS w" row per
 * line (written by :246-247, read by :485/:497). */
int dccm_remap_table_write(const dccm_remap_table *table, const char *path);
int dccm_remap_table_read(const char *path, dccm_remap_table **table);
/* set_mappingTable_interpCoef (common/grid_mapping_util_jones99.f90:446-506):
 * recv_index = iD + GNXR*(jD-1), send_index = iS + GNXS*(jS-1), 1-based. */
int dccm_remap_table_index(const dccm_remap_table *table, int GNXS, int GNXR,
                           int32_t *send_index, int32_t *recv_index, double *coef);
int dccm_remap_table_destroy(dccm_remap_table *table);

/* =====================================================================
 * Remap apply (the jcup interpolation callback)
 * dccm_remap_plan_create takes the operation list of set_operation_index /
 * set_interpolate_coef (common/interpolation_data_latlon_mod.f90:116-270):
 * 1-based send/recv point indices and coefficients, in table order.  It
 * validates every index (the reference reads out of bounds instead) and
 * builds a CSR matrix on the device whose per-row order is the table order.
 * dccm_interpolate_data replaces interpolate_data
 * (common/interpolate_data.f90:1-15 -> interpolate_data_latlon,
 * common/interpolation_data_latlon_mod.f90:274-306): recv_data(:,:) is
 * zeroed and then recv(r,d) += send(s,d)*coef in table order, with the
 * product and the sum rounded separately, so results are bit-identical to
 * the reference loop.  mapping/exchange tags select the plan on the
 * caller's side and are not arguments here.  One call handles
 * n_recv_points * num_of_data < 2^30 destination values; larger calls
 * return DCCM_ERR_UNSUPPORTED (split the fields over several calls).
 * ===================================================================== */
typedef struct dccm_remap_plan dccm_remap_plan;

int dccm_remap_plan_create(int64_t n_send_points, int64_t n_recv_points,
                           int64_t num_of_operation, const int32_t *send_index,
                           const int32_t *recv_index, const double *coef,
                           dccm_remap_plan **plan);
int dccm_remap_plan_destroy(dccm_remap_plan *plan);
int dccm_remap_plan_info(const dccm_remap_plan *plan, int64_t *nnz,
                         int64_t *n_send_points, int64_t *n_recv_points);
/* Host arrays send_data(sn1,sn2), recv_data(rn1,rn2); num_of_data <= sn2, rn2. */
int dccm_interpolate_data(dccm_remap_plan *plan, int64_t sn1, int64_t sn2,
                          const double *send_data, int64_t rn1, int64_t rn2,
                          double *recv_data, int num_of_data);
/* Device arrays; field d of src starts at src + d*ld_src. */
int dccm_remap_apply_dev(dccm_remap_plan *plan, const double *src, int64_t ld_src,
                         double *dst, int64_t ld_dst, int nfields, void *stream);

/* Compensated FP64 global integral sum_i f[i]*area[i] of a device array
 * (IntLonLat_xy, used by atm/dccm_atm_mod.f90:668-669 and
 * ocn/dccm_ocn_mod.f90:803-804; external in the reference).  The result is
 * written to *result (host) after the stream has synchronised. */
int dccm_area_integral_dev(const double *f, const double *area, int64_t n,
                           double *result, void *stream);

/* The same compensated integral without allocating any device memory.
 * No counterpart in the reference: this is for callers that cannot call
 * cudaMalloc, such as a model that has already reserved the whole GPU for
 * its own allocator, so that a component linked into it has no memory
 * left to allocate.  Its scratch is a fixed 256 KB array in the library's
 * device image, held by every GPU that loads the library until the process
 * exits.  Limit: n <= 67,108,864 (2^26) elements, else DCCM_ERR_SHAPE.  All
 * calls share that array, so calls that overlap on the GPU race; serialise
 * them.  The first call in each CUDA context looks up the array's device
 * address (with that context current).  Like dccm_area_integral_dev it
 * copies the result to *result (host) and synchronises the stream before
 * returning. */
int dccm_area_integral_noalloc_dev(const double *f, const double *area, int64_t n,
                                   double *result, void *stream);

/* =====================================================================
 * Spherical-harmonic transforms on the Gaussian grid
 * Replace the SPML transforms that the atmosphere dynamics call through
 * libdcpam5 (atm/dcpam_main_mod.f90:2173-2180) and SPML's w_Initial(nMax,
 * iMax, jMax) with its grid axes xy_Lon, xy_Lat, x_Lon_Weight, y_Lat_Weight
 * (tool/gmapgen/gmapgen_main.f90:262-305).  SPML is external and not
 * vendored, so the convention is this library's own:
 *   - latitudes ascending south to north, mu_j = sin(lat_j) the roots of
 *     P_J, weights w_j with sum 2; longitudes 2 pi i / I;
 *   - Pbar_n^m with integral_{-1}^{1} Pbar^2 dmu = 2, no Condon-Shortley
 *     phase, triangular truncation n <= N = nmax;
 *   - spec[b][k] complex (re, im interleaved doubles), k = idx(m,n) =
 *     m(N+1) - m(m-1)/2 + (n-m) for m = 0..N, n = m..N (Im s_n^0 = 0);
 *   - grid[b][j][i] doubles, i fastest (Fortran (0:imax-1, 1:jmax, b));
 *   - inverse: g = Re F_0 + 2 Re sum_{m>=1} F_m e^{i m lon},
 *     F_m(mu) = sum_n s_n^m Pbar_n^m(mu);
 *   - forward: s_n^m = (1/2) sum_j w_j Pbar_n^m(mu_j) (1/I) sum_i g_ij e^{-i m lon_i}.
 * precision DCCM_SHT_FP64: FP64 throughout (CUDA cores).
 * precision DCCM_SHT_MIXED: Legendre sums on the tensor cores in split
 * BF16 x 3 with FP32 accumulation, FFT in FP32; relative L2 error of a
 * forward(inverse(s)) round trip below 1e-6.  Requires jmax/2 % 16 == 0.
 * precision DCCM_SHT_MIXED_FP16: the same with FP16 operands, each split
 * into hi + lo (22 bits, 3 products instead of 6): the Legendre tables are
 * scaled by a power of two per zonal wavenumber m, the spectra (inverse)
 * and the Fourier coefficients (forward) by a power of two per field-level
 * from the field-level's largest value, so both fit FP16's range; the
 * scales are undone exactly in FP32.  Mixed paths take values within FP32's
 * range.
 * Requirements: jmax even, jmax >= nmax+1, imax > 2 nmax, imax = 32 R with
 * R in {2, 3, 4, 6, 8, 12, 16, 24, 32} (imax = 64 ... 1024).
 * ===================================================================== */
enum { DCCM_SHT_FP64 = 0, DCCM_SHT_MIXED = 1, DCCM_SHT_MIXED_FP16 = 2 };

typedef struct dccm_sht_plan dccm_sht_plan;

int dccm_sht_plan_create(int nmax, int imax, int jmax, int precision, int max_batch,
                         dccm_sht_plan **plan);
int dccm_sht_plan_destroy(dccm_sht_plan *plan);
/* Grid axes as SPML returns them (host arrays, any may be NULL). */
int dccm_sht_axes(const dccm_sht_plan *plan, double *x_Lon, double *y_Lat,
                  double *x_Lon_Weight, double *y_Lat_Weight);
/* Gauss-Legendre nodes mu[jmax] and weights w[jmax] computed on the GPU. */
int dccm_sht_gauss(const dccm_sht_plan *plan, double *mu, double *w);
/* FP64 Pbar table as computed on the GPU: pnm[idx(m,n)*(jmax/2) + jj] at
 * mu[jmax/2 + jj] (northern hemisphere), host array. */
int dccm_sht_pnm(const dccm_sht_plan *plan, double *pnm);
/* Device arrays, stream-ordered; batch <= max_batch field-levels. */
int dccm_sht_inverse_dev(dccm_sht_plan *plan, const double *spec, double *grid, int batch,
                         void *stream);
int dccm_sht_forward_dev(dccm_sht_plan *plan, const double *grid, double *spec, int batch,
                         void *stream);
/* Host arrays; returns after the result is in host memory. */
int dccm_sht_inverse(dccm_sht_plan *plan, const double *spec, double *grid, int batch);
int dccm_sht_forward(dccm_sht_plan *plan, const double *grid, double *spec, int batch);
/* Synchronises the device and reports (then clears) the error flag that
 * bounded device waits set; DCCM_ERR_TIMEOUT if one gave up. */
int dccm_sht_status(dccm_sht_plan *plan, int *device_error);

/* The same transforms in SPML's real spectral layout, the arrays a DCPAM
 * caller holds: SPML's xya_wa (spectral -> grid) and wa_xya (grid ->
 * spectral) of its wa_module, called by the dynamics through libdcpam5
 * (atm/dcpam_main_mod.f90:2173-2180); w_Initial and the axes as above
 * (tool/gmapgen/gmapgen_main.f90:262-305).  wa[b][l] doubles, (N+1)^2 per
 * field-level (Fortran wa((nmax+1)**2, kmax)), l = l_nm(n, m) - 1 =
 * n(n+1) + m for m = -n..n: Re s_n^m at m >= 0, Im s_n^|m| at m < 0.
 * SPML's expansion, normalisation and phase are this library's (above), so
 * the layouts differ by a permutation only; it is restated from SPML's
 * published l_nm / nm_l (SPML is external: unpinned against its code).
 * xya as grid above.  Batch <= max_batch.  The first call on a plan sets up
 * its permutation tables and a spectral buffer of max_batch field-levels
 * (device allocation: make it before any stream capture).  The _dev forms
 * are stream-ordered; the host forms return when the result is in host
 * memory and report DCCM_ERR_TIMEOUT as dccm_sht_inverse does. */
int dccm_sht_xya_wa_dev(dccm_sht_plan *plan, const double *wa, double *xya, int batch, void *stream);
int dccm_sht_wa_xya_dev(dccm_sht_plan *plan, const double *xya, double *wa, int batch, void *stream);
int dccm_sht_xya_wa(dccm_sht_plan *plan, const double *wa, double *xya, int batch);
int dccm_sht_wa_xya(dccm_sht_plan *plan, const double *xya, double *wa, int batch);
/* The permutations alone, device arrays, stream-ordered: SPML wa <-> this
 * library's spec (for callers that feed dccm_step_* or dccm_spec_apply_dev,
 * which take the native layout). */
int dccm_sht_spec_from_wa_dev(dccm_sht_plan *plan, const double *wa, double *spec, int batch, void *stream);
int dccm_sht_wa_from_spec_dev(dccm_sht_plan *plan, const double *spec, double *wa, int batch, void *stream);

/* Ensemble of mixed truncations: ngroups (<= 8) truncation groups, each a
 * plan as above holding the field-levels of all members of that truncation
 * (members of one truncation are concatenated along the batch).  On the
 * mixed path each direction is ONE persistent tensor-core Legendre launch
 * and ONE FFT launch over all groups; the FP64 path runs group by group.
 * spec[g], grid[g] are device pointers of group g; batch[g] <= max_batch[g]. */
typedef struct dccm_sht_ensemble dccm_sht_ensemble;

int dccm_sht_ensemble_create(int ngroups, const int *nmax, const int *imax, const int *jmax,
                             const int *max_batch, int precision, dccm_sht_ensemble **ens);
int dccm_sht_ensemble_destroy(dccm_sht_ensemble *ens);
int dccm_sht_ensemble_inverse_dev(dccm_sht_ensemble *ens, const double *const *spec,
                                  double *const *grid, const int *batch, void *stream);
int dccm_sht_ensemble_forward_dev(dccm_sht_ensemble *ens, const double *const *grid,
                                  double *const *spec, const int *batch, void *stream);
int dccm_sht_ensemble_status(dccm_sht_ensemble *ens, int *device_error);
int dccm_sht_ensemble_groups(const dccm_sht_ensemble *ens, int *ngroups);

/* =====================================================================
 * Coupling step
 * One coupling step of the hot path on one GPU, as one CUDA graph: the
 * atmosphere's inverse then forward transforms of nfl field-levels (the
 * transforms of the dynamics, atm/dcpam_main_mod.f90:2173-2180), and,
 * concurrently, the remap of nfields surface fields (interpolate_data,
 * reached from jcup_get_data at sfc/dccm_sfc_mod.f90:865-881) followed by
 * the bulk flux on the destination grid (sfc/dccm_sfc_mod.f90:886-897).
 * All pointers in the descriptor are device pointers owned by the caller
 * (a_Sig1Info excepted: host, read at creation); a stage whose plan is
 * NULL is left out.  The graph is recorded at creation, so the buffers must
 * stay valid and at the same addresses for the life of the step.
 * ===================================================================== */
/* One remap of a step: nfields fields through one plan.  With nsub > 0 the
 * destination of field f is dst + (f % nsub)*ld_dst + (f / nsub)*ld_dst2
 * (e.g. nsub surface fields of consecutive ensemble members, each member's
 * block ld_dst2 further along the same output arrays); nsub = 0 means
 * dst + f*ld_dst. */
typedef struct dccm_step_remap {
  dccm_remap_plan *plan;
  int nfields;
  const double *src;           /* field f at src + f*ld_src */
  int64_t ld_src;
  double *dst;
  int64_t ld_dst;
  int nsub;
  int64_t ld_dst2;
} dccm_step_remap;

typedef struct dccm_step_desc {
  dccm_sht_plan *sht;          /* transform plan, or NULL */
  int nfl;                     /* field-levels per step (<= plan's max_batch) */
  const double *spec_in;       /* [nfl][ncoef] complex */
  double *grid;                /* [nfl][jmax][imax] */
  double *spec_out;            /* [nfl][ncoef] complex */
  dccm_sht_ensemble *ens;      /* ensemble transforms instead of sht, or NULL */
  const double *const *ens_spec_in;  /* per group, as dccm_sht_ensemble_*_dev */
  double *const *ens_grid;
  double *const *ens_spec_out;
  const int *ens_nfl;
  int nremap;                  /* remaps, run in order before the flux */
  const dccm_step_remap *remaps;
  const dccm_sfc_bulk_flux_args *flux;  /* device arrays, or NULL */
  const dccm_sfc_grid *flux_grid;
  /* Implicit surface coupling around the flux (NULL: none).  The surface
   * branch then runs: the forward sweep (implcpl_fwd's arrays; it writes
   * ImplCplCoef1/2, which `remaps` carry to the flux grid), the remaps,
   * the flux, the remaps_post (e.g. DelVarImplCPL back to level 1 of the
   * tendencies, as the coupler does at atm/dccm_atm_mod.f90:832-835), and
   * the backward sweep on implcpl_fwd's tendencies.  Append-only fields: a
   * caller that zero-initialises the descriptor keeps the plain step. */
  dccm_implcpl *implcpl;
  const dccm_implcpl_forward_args *implcpl_fwd;  /* device arrays */
  int nremap_post;
  const dccm_step_remap *remaps_post;
} dccm_step_desc;

typedef struct dccm_step dccm_step;

/* One host<->device copy of dccm_step_run_host. */
typedef struct dccm_host_copy {
  void *host;
  void *dev;
  size_t bytes;
} dccm_host_copy;

int dccm_step_create(const dccm_step_desc *desc, dccm_step **step);
int dccm_step_destroy(dccm_step *step);
/* Replays the step's graph on stream (stream-ordered, no synchronisation). */
int dccm_step_run(dccm_step *step, void *stream);
/* Runs the stages one after another on stream with events between them and
 * returns their device times: ms[0] Legendre synthesis, ms[1] inverse FFT,
 * ms[2] forward FFT, ms[3] Legendre analysis, ms[4] remaps, ms[5] bulk
 * flux (six floats; with the implicit coupling, ms[4] includes its
 * forward sweep and ms[5] the remaps after the flux and the backward
 * sweep).  Synchronises. */
int dccm_step_run_timed(dccm_step *step, void *stream, float *ms);
/* Copies nh2d host buffers to the device, runs the step, copies nd2h device
 * buffers back and synchronises: the step for a caller whose data live in
 * host memory.  With page-locked host buffers the copies are recorded into
 * a graph of their own (kept until the copy lists change), each next to the
 * stage that needs or produces its data, so that they overlap the kernels:
 * spectral inputs before Legendre synthesis, surface inputs at the head of
 * the remap/flux branch, grid outputs right after the inverse FFT, spectral
 * outputs after the analysis, surface outputs after the flux.  A copy that
 * touches the buffers of both branches, or that reads memory an upload of
 * the same call writes, is ordered before (H2D) or after (D2H) the whole
 * step.  Copies whose host buffers lie back to back (e.g. rows of one host
 * allocation, over 1 MiB in all) move as one copy-engine transfer through a
 * device staging buffer, gathered or scattered on the device; other copies
 * of at most 1 MiB go, per group, through one kernel that reads or writes
 * the host buffers through their device mapping; larger ones are
 * copy-engine transfers.  The uploads of one branch go on the host link
 * before the other's: the branch whose inputs, kernels (as last timed by
 * dccm_step_run_timed or the autotuner) and results would end later goes
 * first (knob "upload_order": 0 this choice, 1 the transforms' inputs
 * first, 2 the surface inputs first; knob "host_path": 1 + a mask of the
 * copy groups moved through the host mapping instead, see
 * dccm_step_autotune_host; both apply when the graph is recorded, and
 * dccm_step_autotune_host chooses them per step by timing).  With pageable buffers: copies in, graph, copies out.
 * A call whose copy lists equal those the graph was recorded with replays
 * it without examining the buffers again: page-locked host buffers must
 * stay allocated and page-locked while the same lists are passed (call
 * dccm_step_host_release after freeing or unpinning one of them). */
int dccm_step_run_host(dccm_step *step, void *stream, const dccm_host_copy *h2d, int nh2d,
                       const dccm_host_copy *d2h, int nd2h);
/* dccm_step_run_host without the final synchronisation: the copies and the
 * step are enqueued on stream and the call returns; the downloads are in
 * host memory once the stream has synchronised (or an event recorded on
 * it after this call has completed).  Page-locked host buffers only
 * (DCCM_ERR_UNSUPPORTED otherwise).  A step's graph runs once at a time:
 * calls on one step are ordered by passing the same stream.  For
 * independent problems (ensemble members, runs, snapshots), each with its
 * own step, device buffers and host buffers, calls on different streams
 * overlap one problem's downloads with the next one's uploads on the
 * host link, which moves data both ways at once. */
int dccm_step_launch_host(dccm_step *step, void *stream, const dccm_host_copy *h2d, int nh2d,
                          const dccm_host_copy *d2h, int nd2h);
/* Sets this step's host-copy choices as dccm_step_autotune_host would:
 * upload_order (0: the process-wide knob), host_path (0: the process-wide
 * knob, else 1 + the copy-group mask) and the flux CTA cap of the host
 * graph (-1: the process-wide knob, 0: the full grid), and drops the
 * recorded host graph.  For a caller that times its own schedule, e.g.
 * two instances in flight, where the copy engines alone (host_path 1)
 * leave the SMs to the other instance's kernels. */
int dccm_step_host_choice(dccm_step *step, int upload_order, int host_path, int flux_ctas);
/* Drops the graph and the staging buffers dccm_step_run_host keeps for its
 * copy lists (the next call records them again). */
int dccm_step_host_release(dccm_step *step);
/* Chooses, for these page-locked copy lists, the upload order (1: the
 * transforms' inputs first, 2: the surface inputs first) and the copy path
 * of each group of copies, host_path = 1 + mask with mask bit 0 the
 * transforms' uploads, bit 1 the surface uploads, bit 2 the transforms'
 * downloads (grid, spectra), bit 3 the surface downloads: a set bit moves
 * the group in one kernel through the host mapping, a clear bit by copy
 * engines with host-contiguous runs through a staging buffer.  Bit 4 (a flux
 * on one interior row, no implicit coupling or remaps after it): the surface
 * copies that are exactly one interior row of a flux input or output are
 * done by the flux kernel itself, which reads those host rows and writes its
 * results to them through their device mapping as it computes the columns
 * (and still fills the device arrays, as the copies would).  It replays the
 * step with each of the 32 combinations (2 interleaved rounds of 6 replays
 * on stream, each after a 256 MB device write; the step's outputs are
 * written as by dccm_step_run_host), keeps the fastest, times it against the
 * same mask with bit 4 under either upload order and keeps the fastest of
 * the three, then times the winner with the flux kernel's full grid against
 * the process-wide "flux_ctas" cap (with host copies the surface results are
 * the first downloads, so the fastest flux can win), then the flux kernel's
 * CTA size for this graph (the process-wide "flux_threads" against 64, 128
 * and 256), and leaves the graph recorded.  chosen (3 ints, may be NULL) receives the order, host_path and
 * the flux CTA cap of this graph (0: the full grid); all 0 with pageable
 * buffers, for which there is nothing to choose.  Each candidate is timed
 * as the caller sees it: host clock from the graph launch to the end of the
 * stream synchronisation (kernels writing host memory through the mapping
 * can finish before their writes land).  ms (32 floats, may be NULL)
 * receives each combination's time per step at index 16 (order - 1) +
 * mask.  The process-wide knobs "upload_order", "host_path" and "flux_ctas"
 * (dccm_tune_set) apply to steps that have not been tuned this way. */
int dccm_step_autotune_host(dccm_step *step, void *stream, const dccm_host_copy *h2d, int nh2d,
                            const dccm_host_copy *d2h, int nd2h, int *chosen, float *ms);

/* Autotuner: chooses the launch shapes of the step's kernels by timing
 * candidates of each knob on the stage it affects ("tc_shape": 0 runs the
 * tensor-core Legendre kernel one CTA an SM with two load stages and eight
 * epilogue warps, 1 runs it two CTAs an SM with one load stage and four
 * epilogue warps where its tables allow (N tiles of at most 64 rows, e.g.
 * up to T85 on its Gaussian grid); "tc_ctas": persistent CTAs of
 * that kernel, at most one wave, "fft_rpw": row pairs per FFT warp for
 * rows of one warp (I <= 384; 1 or 2, in turn), "fft_bb": warps per FFT CTA
 * (4, 8 or 16), "flux_threads", "remap_threads": CTA sizes, "remap_fc":
 * fields per thread of the remap, 1, 2, 3, 4 or 6), then "serial"
 * (1: ordinary launches instead of programmatic dependent launches along
 * the transform chain), "tc_ctas" again, "prio" (0: every kernel at the
 * launching stream's priority; 1: the transform chain's, 2: the remaps'
 * and the flux's kernels at the device's greatest priority, so that SMs
 * freed while both branches have CTAs waiting go to that branch first),
 * and, with a flux, "prio", "flux_threads" and "flux_ctas" (CTA cap of the
 * flux kernel's grid, 0: 16 per SM) together (3 x 3 x 4 candidates), on
 * replays of the whole step graph,
 * where the two branches run concurrently; applies the winners and
 * records the step's graph again.  Every timed run follows a 256 MB
 * device write, so that the step finds L2 as it does between the model's
 * other work.  With cache_path the choice is read
 * from / appended to that file (one JSON object per line, keyed by the
 * GPU name and SM count and the step's shapes).  chosen (4 ints, may be
 * NULL) receives tc_ctas, fft_bb, flux_threads, remap_threads (read
 * "serial", "prio", "flux_ctas", "remap_fc", "tc_shape" and "fft_rpw" with dccm_tune_get).  The knobs are
 * process-wide defaults of later launches too. */
int dccm_step_autotune(dccm_step *step, const char *cache_path, int *chosen);
/* Process-wide knobs of later launches (and of graphs recorded later): the
 * launch shapes above, "upload_order" and "host_path" (dccm_step_run_host),
 * and two of the failure path: "wait_limit_ms", the limit of every bounded
 * wait of the tensor-core Legendre kernel (0: 1000 ms; at most 60000), and
 * "tc_withhold_loads" (1: that kernel's load thread issues no copies, so
 * that its waits expire and the call reports DCCM_ERR_TIMEOUT through
 * dccm_sht_status / the host entry points; nothing is left in flight, and
 * the next launch with the knob at 0 is unaffected: a test of the timeout
 * path, never for production).  Unknown knob or value: DCCM_ERR_INVALID_ARG. */
int dccm_tune_set(const char *knob, int value);
int dccm_tune_get(const char *knob, int *value);

/* ------------------------------------------------------------------
 * Spectral-space operators around the transform (the reference applies
 * them inside DynamicsHSplVAS83, atm/dcpam_main_mod.f90:2173-2180, from
 * the external dcpam5 library; HDOrder and the e-folding time of the
 * largest wavenumber: exp/APEI07Couple/common/dcpam/
 * dcpam_APEI07Couple_T21L16.conf:205-227).  Built from the mathematics;
 * every operator scales coefficient (m, n) of [batch][ncoef] complex
 * spectra (the SHT layout) by a factor f_n of the total wavenumber:
 *   DCCM_SPEC_LAPLACIAN        -n(n+1)/a^2
 *   DCCM_SPEC_INV_LAPLACIAN    -a^2/(n(n+1)), 0 for n = 0
 *   DCCM_SPEC_HDIFF_TENDENCY   -D_n
 *   DCCM_SPEC_HDIFF_IMPLICIT   1/(1 + dt D_n)  (backward step over dt)
 * with D_n = nu (K_n - c), K_n = (n(n+1)/a^2)^(order/2), c = K_1 when
 * rotation_correction is set (rigid rotation is not damped) else 0,
 * D_0 = 0 (the global mean is never diffused), and
 * nu = 1/(efold_time (K_N - c)).  a = radius.  spec_in may equal spec_out.
 * nmax < 2048 (DCCM_ERR_UNSUPPORTED above).
 * ------------------------------------------------------------------ */
#define DCCM_SPEC_LAPLACIAN 0
#define DCCM_SPEC_INV_LAPLACIAN 1
#define DCCM_SPEC_HDIFF_TENDENCY 2
#define DCCM_SPEC_HDIFF_IMPLICIT 3
typedef struct dccm_spec_op {
  int kind;                /* DCCM_SPEC_* */
  double radius;           /* planet radius a (m) */
  int order;               /* hyperdiffusion order (even, 2..32), e.g. HDOrder = 8 */
  double efold_time;       /* e-folding time of wavenumber nmax (s) */
  double dt;               /* time step of the implicit form (s) */
  int rotation_correction; /* 1: D_1 = 0 */
} dccm_spec_op;
/* Device arrays, stream-ordered. */
int dccm_spec_apply_dev(int nmax, const dccm_spec_op *op, const double *spec_in, double *spec_out, int batch,
                        void *stream);
/* Host arrays (staged through the device), synchronises. */
int dccm_spec_apply(int nmax, const dccm_spec_op *op, const double *spec_in, double *spec_out, int batch);

/* Measures the device's FP64 FMA throughput (TFLOP/s, best of 5 launches
 * of independent DFMA chains on every SM; synchronises): the denominator
 * of the FP64-bound kernels' roofline fractions. */
int dccm_fp64_peak(void *stream, double *tflops);

/* The bulk-flux kernel's FP64 reciprocal, exp, log, square root and
 * reciprocal square root (fewer FP64 operations than the correctly rounded
 * library calls; within about 2 units in the last place) evaluated
 * elementwise on device arrays, y[i] = f(x[i]), stream-ordered: the entry
 * point their accuracy tests call. */
#define DCCM_FP64_RCP 0
#define DCCM_FP64_EXP 1
#define DCCM_FP64_LOG 2
#define DCCM_FP64_SQRT 3
#define DCCM_FP64_RSQRT 4
int dccm_fp64_fn_dev(int fn, const double *x, double *y, int64_t n, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* DCCM_GB300_H */
