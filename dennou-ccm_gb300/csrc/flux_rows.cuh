// The bulk flux kernel's per-column rows, and the table that binds some of
// them to page-locked host memory.
//
// A row is one interior row (array, slot) of a grid with a single interior
// row (JS = JE: the coupler's list of ocean columns, IA = columns + 2,
// JA = 3).  Bound inputs are read from the host row through its device
// mapping and mirrored into the device row; bound outputs are written to
// the device row and to the host row.  The device arrays thus hold what
// copies before and after the kernel would have left there, while the
// host link carries the data as the columns are computed
// (dccm_step_run_host, host_path bit 4).
#pragma once

#include "dccm_gb300.h"

namespace dccm {
namespace flux {

enum InRow {
  I_ICE, I_PS, I_TA, I_Q1, I_U, I_V, I_ZS, I_SDW, I_LDW,
  I_TS,               // SfcTemp slots 1, 2
  I_ALB = I_TS + 2,   // SfcAlbedo slots 1, 2
  I_C1 = I_ALB + 2,   // ImplCplCoef1 slots 1-4
  I_C2 = I_C1 + 4,    // ImplCplCoef2 slots 1-4
  NIN = I_C2 + 4
};
enum OutRow {
  O_DELV,              // DelVarImplCPL slots 1-4
  O_FNS = O_DELV + 4,  // SfcHFlx_ns slots 1, 2
  O_FSR = O_FNS + 2,   // SfcHFlx_sr slots 1, 2
  O_DFDT = O_FSR + 2,  // DSfcHFlxDTs slots 1, 2
  O_WSX = O_DFDT + 2,  // the ten 3-slot outputs follow
  O_WSY = O_WSX + 3,
  O_SEN = O_WSY + 3,
  O_QV = O_SEN + 3,
  O_LAT = O_QV + 3,
  O_CVEL = O_LAT + 3,
  O_CTEMP = O_CVEL + 3,
  O_CQ = O_CTEMP + 3,
  O_SUW = O_CQ + 3,
  O_LUW = O_SUW + 3,
  O_TS3 = O_LUW + 3,  // SfcTemp slot 3
  O_ALB3,             // SfcAlbedo slot 3
  NOUT
};

struct HostRows {
  const double *in[NIN];  // host row (device address) read in place of the device row
  double *din[NIN];       // the device row it is mirrored into
  double *out[NOUT];      // host row (device address) written besides the device row
  int any;
};

// First element of the interior row of (array base, slot) on the grid.
inline double *row_start(const void *base, const dccm_sfc_grid &g, int slot) {
  const int64_t plane = (int64_t)g.IA * g.JA;
  return (double *)base + slot * plane + (int64_t)g.IA * (g.JS - 1) + (g.IS - 1);
}
// Device row of input row k / output row k.
double *in_row(const dccm_sfc_bulk_flux_args &a, const dccm_sfc_grid &g, int k);
double *out_row(const dccm_sfc_bulk_flux_args &a, const dccm_sfc_grid &g, int k);
// The flux on a stream with host rows bound (h may be null).
int launch_rows(const dccm_sfc_bulk_flux_args *a, const dccm_sfc_grid *g, const HostRows *h, cudaStream_t s);

}  // namespace flux
}  // namespace dccm
