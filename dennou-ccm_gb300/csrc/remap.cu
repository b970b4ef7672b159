// Jones-99 remap: table generator (GPU), table file I/O, CSR apply kernel,
// and the compensated area integral.
//
// Reference: common/grid_mapping_util_jones99.f90 (generator :35-442, reader
// :446-506) and common/interpolation_data_latlon_mod.f90:274-306 (apply).
//
// Generator.  The reference loops over destination cells; per cell it scans
// source edges linearly and writes the rows whose |w| > 1e-14.  The range
// search depends only on the destination column (longitude) or row
// (latitude), so it is done once per column and per row on the host, in the
// reference's call order, which also reproduces its stale-value behaviour
// (SrcRangeX(2) and SrcRangeY(1) keep the previous call's value when no
// source edge matches).  Cell edges are built on the host by the
// reference's sequential asin recurrence (:142-151), so every comparison of
// the search sees the same doubles as the reference.  The sines of all
// edges are tabulated there too, and the GPU evaluates the weights of all
// cells in parallel with separately rounded operations in the reference's
// order: REF-mode weights are bit-identical to the restated reference.
//
// Apply.  The table is grouped by destination, so a stable counting sort
// groups it by row without changing the per-row order.  The rows are then
// stored as a sliced ELL matrix: slices of 32 destination rows (one warp),
// each slice as many record columns wide as its longest row, record k of
// lane r at slice_base + 32 k + r, so that a warp's k-th records are one
// coalesced 512-byte load.  Within each window of 256 consecutive rows the
// rows are ordered by length (stable) before they are cut into slices, so
// that a slice's rows are about equally long: the padding records, which
// cost FP64 instructions like real ones, fall from 19 % to 5 % of the
// records at c3 (17 % to 3 % at c5); each lane reads its row number from
// the plan.  A record is 16 bytes (weight, source
// column; column -1 pads a short row).  One thread owns a destination row
// and FC of the fields: it loads each record once and gathers the FC source
// values of its column (all of a round's gathers in flight together);
// sums start at zero and add the separately rounded products in table
// order, which makes the result bit-identical to the reference loop
// (:293-302); the first addition of a row, 0 + p, is p with -0 turned into
// +0, which integer instructions give exactly without the FP64 pipe (the
// pipe the kernel is bound by: one DMUL per entry and field, one DADD per
// entry after the first).
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "remap_table.cuh"
#include "common.cuh"
#include "nvtx.cuh"


struct dccm_remap_plan {
  int64_t n_send = 0, n_recv = 0, nnz = 0;
  int64_t nslice = 0, nrec = 0;  // 32-row slices; records including padding
  int2 *d_slices = nullptr;      // per slice: (first record / 32, width in records)
  int *d_rows = nullptr;         // per slice lane: its destination row (0-based), -1 past the last
  double2 *d_ent = nullptr;      // nrec records: x = weight, y = column (0-based, -1 pad) bits
  dccm::DevBuf stage;            // host entry point staging
  cudaStream_t stream = nullptr;
};

namespace dccm {
namespace remap {

constexpr int UNSET = -2147483647;

// ---------------------------------------------------------------- apply
// Thread = destination row r (lane of its slice, rows[]) x fields f0 .. f0+FC-1
// (f0 = FC blockIdx.y).  Field f is read at src + f ld_src and written at
// (f % nsub) ld_dst + (f / nsub) ld_dst2.  U records a round: their loads,
// then their U x FC source gathers, are in flight before the in-order sums.
template <int FC>
__global__ void __launch_bounds__(256)
sell_apply(const int2 *__restrict__ slices, const int *__restrict__ rows, const double2 *__restrict__ ent,
           const double *__restrict__ src, int64_t ld_src, double *__restrict__ dst, int64_t ld_dst, int nslice,
           int nfields, int nsub, int64_t ld_dst2) {
  constexpr int U = FC >= 6 ? 2 : 4;
  const int lane = threadIdx.x & 31;
  const int sl_i = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  if (sl_i >= nslice) return;
  const int f0 = blockIdx.y * FC;
  const int r = __ldg(rows + sl_i * 32 + lane);
  const int2 sl = __ldg(slices + sl_i);
  const double2 *e = ent + (int64_t)sl.x * 32 + lane;
  const double *sp[FC];
#pragma unroll
  for (int f = 0; f < FC; ++f) sp[f] = src + (int64_t)(f0 + f < nfields ? f0 + f : f0) * ld_src;
  double acc[FC];
#pragma unroll
  for (int f = 0; f < FC; ++f) acc[f] = 0.0;
  for (int k0 = 0; k0 < sl.y; k0 += U) {
    double2 q[U];
#pragma unroll
    for (int u = 0; u < U; ++u)
      q[u] = k0 + u < sl.y ? __ldg(e + (int64_t)(k0 + u) * 32) : make_double2(0.0, __longlong_as_double(-1LL));
    double x[U][FC];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const long long c = __double_as_longlong(q[u].y);
#pragma unroll
      for (int f = 0; f < FC; ++f) x[u][f] = (c >= 0 && f0 + f < nfields) ? __ldg(sp[f] + c) : 0.0;
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (__double_as_longlong(q[u].y) < 0) continue;
      if (u == 0 && k0 == 0) {
        // the row's first entry: 0 + p, which is p except that -0 becomes +0;
        // done on the integer pipes (the FP64 pipe is this kernel's limit)
#pragma unroll
        for (int f = 0; f < FC; ++f) {
          const double pr = __dmul_rn(x[u][f], q[u].x);
          acc[f] = (__double_as_longlong(pr) << 1) == 0 ? 0.0 : pr;
        }
      } else {
#pragma unroll
        for (int f = 0; f < FC; ++f) acc[f] = __dadd_rn(acc[f], __dmul_rn(x[u][f], q[u].x));
      }
    }
  }
  if (r < 0) return;
#pragma unroll
  for (int f = 0; f < FC; ++f) {
    const int fg = f0 + f;
    if (fg >= nfields) break;
    const int fs = fg / nsub;
    dst[(int64_t)(fg - fs * nsub) * ld_dst + (int64_t)fs * ld_dst2 + r] = acc[f];
  }
}

int apply2(dccm_remap_plan *p, const double *src, int64_t ld_src, double *dst, int64_t ld_dst, int nfields,
           int nsub, int64_t ld_dst2, cudaStream_t s) {
  if (p->n_recv == 0 || nfields == 0) return DCCM_OK;
  if (p->n_recv >= (1LL << 31) - 32) return DCCM_ERR_UNSUPPORTED;
  if (nsub <= 0) {
    nsub = nfields;
    ld_dst2 = 0;
  }
  int threads = tunables().remap_threads > 0 ? tunables().remap_threads : 128;
  threads = threads < 32 ? 32 : (threads > 256 ? 256 : threads / 32 * 32);
  int fc = tunables().remap_fc > 0 ? tunables().remap_fc : (nfields >= 6 ? 3 : nfields);
  fc = fc >= 6 ? 6 : (fc >= 4 ? 4 : (fc >= 3 ? 3 : (fc >= 2 ? 2 : 1)));
  const int64_t blocks = (p->nslice * 32 + threads - 1) / threads;
  const int64_t ychunks = (nfields + fc - 1) / fc;
  if (blocks > 0x7FFFFFFF || ychunks > 65535) return DCCM_ERR_UNSUPPORTED;
  const dim3 grid((unsigned)blocks, (unsigned)ychunks);
  const int ns = (int)p->nslice;
#define DCCM_SELL(FC_)                                                                                   \
  DCCM_CUDA(launch_surface(sell_apply<FC_>, grid, dim3(threads), 0, s, (const int2 *)p->d_slices,          \
                           (const int *)p->d_rows, (const double2 *)p->d_ent, src, ld_src, dst, ld_dst, ns, \
                           nfields, nsub, ld_dst2))
  switch (fc) {
    case 6: DCCM_SELL(6); break;
    case 4: DCCM_SELL(4); break;
    case 3: DCCM_SELL(3); break;
    case 2: DCCM_SELL(2); break;
    default: DCCM_SELL(1); break;
  }
#undef DCCM_SELL
  DCCM_LAUNCH_CHECK();
  return DCCM_OK;
}

int apply(dccm_remap_plan *p, const double *src, int64_t ld_src, double *dst, int64_t ld_dst,
          int nfields, cudaStream_t s) {
  return apply2(p, src, ld_src, dst, ld_dst, nfields, 0, 0, s);
}

// ------------------------------------------------------------ generator
struct HaloGrid {
  int nx = 0, ny = 0;
  std::vector<double> x, u, y, v;  // 1-based with halo, as in the reference
};

// gen_gridmapfile_lonlat2lonlat + calc_edge_coordinate (:78-152).
static void make_grid(HaloGrid &g, const double *lon, int nx, const double *lat, int ny,
                      const double *latwt) {
  const double PI = acos(-1.0);
  const int IA = nx + 2, IS = 2, IE = IA - 1;
  const int JA = ny + 2, JS = 2, JE = JA - 1;
  g.nx = nx;
  g.ny = ny;
  g.x.assign(IA + 2, 0.0);
  g.u.assign(IA + 2, 0.0);
  g.y.assign(JA + 2, 0.0);
  g.v.assign(JA + 2, 0.0);
  for (int i = IS; i <= IE; ++i) g.x[i] = lon[i - IS];
  for (int j = JS; j <= JE; ++j) g.y[j] = lat[j - JS];
  g.x[IS - 1] = g.x[IE] - 2.0 * PI;
  g.x[IE + 1] = g.x[IS] + 2.0 * PI;
  for (int i = IS - 1; i <= IE; ++i) g.u[i] = 0.5 * (g.x[i] + g.x[i + 1]);
  g.v[JS - 1] = -PI / 2.0;
  for (int j = JS; j <= JE - 1; ++j) g.v[j] = asin(latwt[j - JS] + sin(g.v[j - 1]));
  g.v[JE] = PI / 2.0;
}

// Per-launch constants of the weight kernel.
struct GenParams {
  int nxd, nyd, nxs, nys;
  int mode, order;
  double DLon_k, DLon_nk, DLon_n;
  const int *x0, *x1;          // per destination column: source column range (halo index)
  const int *y0, *y1;          // per destination row: source row range (halo index)
  const double *sinS, *sinD;   // sin of source / destination latitude edges (halo index)
  const double *hS, *hD;       // cos(v) + v sin(v) of the edges (second order)
  const double *vS, *vD;       // latitude edges
  const double *yS;            // source centre latitudes (halo index)
  const double *uS, *uD;       // longitude edges
  const uint8_t *mask;         // destination mask or null
  const int *lptr, *lidx;      // conservative mode: source columns per destination column
  const double *lov;           // conservative mode: their longitude overlaps
  const int64_t *offs;         // output offsets (fill pass)
  int *cnt;                    // row counts (count pass)
  int32_t *oiD, *ojD, *oiS, *ojS;
  double *ow;
};

// One thread per destination cell; pass 0 counts rows, pass 1 writes them.
template <int PASS>
__global__ void j99_cells(GenParams P) {
  const int64_t ncell = (int64_t)P.nxd * P.nyd;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < ncell;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int iDo = (int)(t % P.nxd), jDo = (int)(t / P.nxd);  // 0-based
    const int iD = iDo + 2, jD = jDo + 2;                      // halo index
    int64_t out = PASS == 1 ? P.offs[t] : 0;
    int count = 0;
    if (P.mask && P.mask[t] == 0) {
      if (PASS == 0) P.cnt[t] = 0;
      continue;
    }
    const int X0 = P.x0[iDo], X1 = P.x1[iDo];
    const int Y0 = P.y0[jDo], Y1 = P.y1[jDo];
    const int NXr = X1 - X0 + 1, NYr = Y1 - Y0 + 1;
    if ((P.mode == 1 || NXr > 0) && NYr > 0) {
      const double sin_k1 = P.sinD[jD - 1], sin_k2 = P.sinD[jD];
      double Ak, dlon_k = 0.0;
      if (P.mode == 0) {
        Ak = __dmul_rn(__dsub_rn(sin_k2, sin_k1), P.DLon_k);
      } else {
        dlon_k = __dsub_rn(P.uD[iD], P.uD[iD - 1]);
        Ak = __dmul_rn(__dsub_rn(sin_k2, sin_k1), dlon_k);
      }
      const int M = (P.mode == 0) ? NXr : (P.lptr[iDo + 1] - P.lptr[iDo]);
      for (int m = 1; m <= M; ++m) {
        int iS;
        double lonw;
        if (P.mode == 0) {
          iS = X0 + m - 1;
          lonw = P.DLon_nk;
        } else {
          iS = P.lidx[P.lptr[iDo] + m - 1];
          lonw = P.lov[P.lptr[iDo] + m - 1];
        }
        for (int n = 1; n <= NYr; ++n) {
          const int jS = Y0 + n - 1;
          // Segment edges: a_AkSegLat (:334-338).
          const double s1 = (n == 1) ? sin_k1 : P.sinS[Y0 + n - 2];
          const double s2 = (n == NYr) ? sin_k2 : P.sinS[Y0 + n - 1];
          const double w1 = __ddiv_rn(__dmul_rn(lonw, __dsub_rn(s2, s1)), Ak);
          if (fabs(w1) > 1e-14) {
            if (PASS == 1) {
              P.oiD[out] = iD - 1; P.ojD[out] = jD - 1;
              P.oiS[out] = iS - 1; P.ojS[out] = jS - 1;
              P.ow[out] = w1;
              ++out;
            }
            ++count;
          }
          if (P.order > 1 && P.mode == 0) {
            // Second-order terms (:252-268, :354-365).
            const double h1 = (n == 1) ? P.hD[jD - 1] : P.hS[Y0 + n - 2];
            const double h2 = (n == NYr) ? P.hD[jD] : P.hS[Y0 + n - 1];
            const double hn1 = P.hS[Y0 + n - 2], hn2 = P.hS[Y0 + n - 1];
            const double sn1 = P.sinS[Y0 + n - 2], sn2 = P.sinS[Y0 + n - 1];
            const double An = __dmul_rn(__dsub_rn(sn2, sn1), P.DLon_n);
            const double ta = __ddiv_rn(__dmul_rn(__dsub_rn(h2, h1), P.DLon_nk), Ak);
            const double tb = __ddiv_rn(
                __dmul_rn(__dmul_rn(__dsub_rn(hn2, hn1), P.DLon_n), w1), An);
            const double w2 = __dsub_rn(ta, tb);
            if (fabs(w2) > 1e-14) {
              const int JSS = 2, JES = P.nys + 1;
              int j1, j2;
              if (jS == JSS) { j1 = jS; j2 = jS + 1; }
              else if (jS == JES) { j1 = jS - 1; j2 = jS; }
              else { j1 = jS - 1; j2 = jS + 1; }
              const double DLat = __dsub_rn(P.yS[j2], P.yS[j1]);
              if (PASS == 1) {
                P.oiD[out] = iD - 1; P.ojD[out] = jD - 1; P.oiS[out] = iS - 1;
                P.ojS[out] = j1 - 1; P.ow[out] = __ddiv_rn(-w2, DLat);
                ++out;
                P.oiD[out] = iD - 1; P.ojD[out] = jD - 1; P.oiS[out] = iS - 1;
                P.ojS[out] = j2 - 1; P.ow[out] = __ddiv_rn(w2, DLat);
                ++out;
              }
              count += 2;
            }
          }
        }
      }
    }
    if (PASS == 0) P.cnt[t] = count;
  }
}

template <typename T>
static int upload(T **d, const std::vector<T> &h) {
  *d = nullptr;
  if (h.empty()) return DCCM_OK;
  DCCM_CUDA(cudaMalloc((void **)d, h.size() * sizeof(T)));
  DCCM_CUDA(cudaMemcpy(*d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
  return DCCM_OK;
}

struct DevFree {
  std::vector<void *> ptrs;
  ~DevFree() {
    for (void *p : ptrs)
      if (p) cudaFree(p);
  }
};

// Periodic overlap of [a1,a2] with [b1,b2], computed on the host.
static double lon_overlap_host(double a1, double a2, double b1, double b2) {
  const double PI_ = 3.141592653589793238462643383279502884;
  double tot = 0.0;
  for (int s = -1; s <= 1; ++s) {
    const double sh = 2.0 * PI_ * s;
    const double lo = a1 > b1 + sh ? a1 : b1 + sh;
    const double hi = a2 < b2 + sh ? a2 : b2 + sh;
    if (hi > lo) tot += hi - lo;
  }
  return tot;
}

int generate(const double *lonS, int nxs, const double *latS, int nys, const double *lonD,
             int nxd, const double *latD, int nyd, const double *latwtS, const double *latwtD,
             int order, int mode, const uint8_t *mask, dccm_remap_table *tab) {
  const double PI = acos(-1.0);
  HaloGrid S, D;
  make_grid(S, lonS, nxs, latS, nys, latwtS);
  make_grid(D, lonD, nxd, latD, nyd, latwtD);
  const int ISS = 2, IES = nxs + 1, JSS = 2, JES = nys + 1;
  const int ISD = 2, IED = nxd + 1, JSD = 2, JED = nyd + 1;
  const int NXD = IED - ISD + 1, NXS = IES - ISS + 1;

  // search_OverwrapRange (:402-438).  The longitude range depends only on
  // iD and the latitude range only on jD, so the first destination row is
  // searched for every column and the other rows for their first column
  // only, keeping the reference's call order for the values it carries over
  // between calls (SrcRangeX(2), SrcRangeY(1)).  A carried value is only
  // needed where nothing matches; on the first call there is none and the
  // grid is refused, as the reference would read an unset value there.
  std::vector<int> X0(nxd), X1(nxd), Y0(nyd), Y1(nyd);
  int rx2 = UNSET, ry1 = UNSET;
  auto searchY = [&](int jD) -> int {
    const double DY1 = D.v[jD - 1], DY2 = D.v[jD];
    int ry2 = -1;
    for (int j = JSS; j <= JES; ++j) {
      if (S.v[j - 1] <= DY1 && DY1 <= S.v[j]) ry1 = j;
      if (S.v[j - 1] <= DY2 && DY2 <= S.v[j]) { ry2 = j; break; }
    }
    if (ry1 == UNSET || ry1 < 0 || ry2 < 0) return DCCM_ERR_SEARCH;
    Y0[jD - JSD] = ry1;
    Y1[jD - JSD] = ry2;
    return DCCM_OK;
  };
  for (int iD = ISD; iD <= IED; ++iD) {
    const double DX1 = D.u[iD - 1], DX2 = D.u[iD];
    int rx1 = -1;
    if (NXS == 1 && NXD != 1) {
      rx1 = ISS; rx2 = ISS;
    } else if (NXS != 1 && NXD == 1) {
      rx1 = ISS; rx2 = IES;
    } else {
      for (int i = ISS; i <= IES; ++i) {
        if (S.u[i - 1] <= DX1 && DX1 <= S.u[i]) rx1 = i;
        if (S.u[i - 1] <= DX2 && DX2 <= S.u[i]) { rx2 = i; break; }
      }
    }
    DCCM_TRY(searchY(JSD));
    if (rx2 == UNSET) return DCCM_ERR_SEARCH;
    X0[iD - ISD] = rx1;
    X1[iD - ISD] = rx2;
  }
  for (int jD = JSD + 1; jD <= JED; ++jD) DCCM_TRY(searchY(jD));

  // Conservative variant: per destination column, the source columns with
  // positive periodic overlap, in ascending order, and the overlaps.
  std::vector<int> lptr(1, 0), lidx;
  std::vector<double> lov;
  if (mode == 1) {
    for (int iD = ISD; iD <= IED; ++iD) {
      const double DX1 = D.u[iD - 1], DX2 = D.u[iD];
      if (NXS == 1) {
        lidx.push_back(ISS);
        lov.push_back(DX2 - DX1);
      } else {
        for (int i = ISS; i <= IES; ++i) {
          const double o = lon_overlap_host(DX1, DX2, S.u[i - 1], S.u[i]);
          if (o > 0.0) {
            lidx.push_back(i);
            lov.push_back(o);
          }
        }
      }
      lptr.push_back((int)lidx.size());
    }
  }

  // Edge tables (halo-indexed) with the host libm, as the reference computes them.
  std::vector<double> sinS(S.v.size()), sinD(D.v.size()), hS(S.v.size()), hD(D.v.size());
  for (size_t k = 0; k < S.v.size(); ++k) {
    sinS[k] = sin(S.v[k]);
    hS[k] = cos(S.v[k]) + S.v[k] * sin(S.v[k]);
  }
  for (size_t k = 0; k < D.v.size(); ++k) {
    sinD[k] = sin(D.v[k]);
    hD[k] = cos(D.v[k]) + D.v[k] * sin(D.v[k]);
  }

  GenParams P = {};
  P.nxd = nxd; P.nyd = nyd; P.nxs = nxs; P.nys = nys;
  P.mode = mode; P.order = order;
  P.DLon_k = 2.0 * PI / (double)NXD;
  if (NXD == 1) { P.DLon_nk = 2.0 * PI / (double)NXS; P.DLon_n = P.DLon_nk; }
  else { P.DLon_nk = 2.0 * PI / (double)NXD; P.DLon_n = 2.0 * PI; }

  DevFree keep;
  int *dX0, *dX1, *dY0, *dY1;
  double *dsinS, *dsinD, *dhS, *dhD, *dvS, *dvD, *dyS, *duS, *duD;
  uint8_t *dmask = nullptr;
  DCCM_TRY(upload(&dX0, X0)); keep.ptrs.push_back(dX0);
  DCCM_TRY(upload(&dX1, X1)); keep.ptrs.push_back(dX1);
  DCCM_TRY(upload(&dY0, Y0)); keep.ptrs.push_back(dY0);
  DCCM_TRY(upload(&dY1, Y1)); keep.ptrs.push_back(dY1);
  DCCM_TRY(upload(&dsinS, sinS)); keep.ptrs.push_back(dsinS);
  DCCM_TRY(upload(&dsinD, sinD)); keep.ptrs.push_back(dsinD);
  DCCM_TRY(upload(&dhS, hS)); keep.ptrs.push_back(dhS);
  DCCM_TRY(upload(&dhD, hD)); keep.ptrs.push_back(dhD);
  DCCM_TRY(upload(&dvS, S.v)); keep.ptrs.push_back(dvS);
  DCCM_TRY(upload(&dvD, D.v)); keep.ptrs.push_back(dvD);
  DCCM_TRY(upload(&dyS, S.y)); keep.ptrs.push_back(dyS);
  DCCM_TRY(upload(&duS, S.u)); keep.ptrs.push_back(duS);
  DCCM_TRY(upload(&duD, D.u)); keep.ptrs.push_back(duD);
  const int64_t ncell = (int64_t)nxd * nyd;
  if (mask) {
    std::vector<uint8_t> hm(mask, mask + ncell);
    DCCM_TRY(upload(&dmask, hm));
    keep.ptrs.push_back(dmask);
  }
  P.x0 = dX0; P.x1 = dX1; P.y0 = dY0; P.y1 = dY1;
  P.sinS = dsinS; P.sinD = dsinD; P.hS = dhS; P.hD = dhD; P.vS = dvS; P.vD = dvD;
  P.yS = dyS; P.uS = duS; P.uD = duD; P.mask = dmask;
  if (mode == 1) {
    int *dlptr, *dlidx;
    double *dlov;
    DCCM_TRY(upload(&dlptr, lptr)); keep.ptrs.push_back(dlptr);
    DCCM_TRY(upload(&dlidx, lidx)); keep.ptrs.push_back(dlidx);
    DCCM_TRY(upload(&dlov, lov)); keep.ptrs.push_back(dlov);
    P.lptr = dlptr; P.lidx = dlidx; P.lov = dlov;
  }

  int *dcnt = nullptr;
  DCCM_CUDA(cudaMalloc(&dcnt, ncell * sizeof(int)));
  keep.ptrs.push_back(dcnt);
  P.cnt = dcnt;
  const int threads = 256;
  int64_t blocks = std::min<int64_t>((ncell + threads - 1) / threads, (int64_t)sm_count() * 16);
  if (blocks < 1) blocks = 1;
  j99_cells<0><<<(unsigned)blocks, threads>>>(P);
  DCCM_LAUNCH_CHECK();
  std::vector<int> cnt(ncell);
  DCCM_CUDA(cudaMemcpy(cnt.data(), dcnt, ncell * sizeof(int), cudaMemcpyDeviceToHost));
  std::vector<int64_t> offs(ncell);
  int64_t total = 0;
  for (int64_t t = 0; t < ncell; ++t) { offs[t] = total; total += cnt[t]; }
  int64_t *doffs;
  DCCM_TRY(upload(&doffs, offs)); keep.ptrs.push_back(doffs);
  P.offs = doffs;
  tab->iD.resize(total); tab->jD.resize(total); tab->iS.resize(total); tab->jS.resize(total);
  tab->w.resize(total);
  if (total > 0) {
    int32_t *o4;
    double *ow;
    DCCM_CUDA(cudaMalloc(&o4, total * 4 * sizeof(int32_t)));
    keep.ptrs.push_back(o4);
    DCCM_CUDA(cudaMalloc(&ow, total * sizeof(double)));
    keep.ptrs.push_back(ow);
    P.oiD = o4; P.ojD = o4 + total; P.oiS = o4 + 2 * total; P.ojS = o4 + 3 * total; P.ow = ow;
    j99_cells<1><<<(unsigned)blocks, threads>>>(P);
    DCCM_LAUNCH_CHECK();
    DCCM_CUDA(cudaMemcpy(tab->iD.data(), P.oiD, total * 4, cudaMemcpyDeviceToHost));
    DCCM_CUDA(cudaMemcpy(tab->jD.data(), P.ojD, total * 4, cudaMemcpyDeviceToHost));
    DCCM_CUDA(cudaMemcpy(tab->iS.data(), P.oiS, total * 4, cudaMemcpyDeviceToHost));
    DCCM_CUDA(cudaMemcpy(tab->jS.data(), P.ojS, total * 4, cudaMemcpyDeviceToHost));
    DCCM_CUDA(cudaMemcpy(tab->w.data(), P.ow, total * 8, cudaMemcpyDeviceToHost));
  }
  return DCCM_OK;
}

// ------------------------------------------------------- area integral
// Error-free transformation a + b = s + e.
__device__ __forceinline__ void two_sum(double a, double b, double &s, double &e) {
  s = __dadd_rn(a, b);
  const double bb = __dsub_rn(s, a);
  e = __dadd_rn(__dsub_rn(a, __dsub_rn(s, bb)), __dsub_rn(b, bb));
}

__device__ __forceinline__ void acc_pair(double &s, double &c, double x) {
  double e;
  two_sum(s, x, s, e);
  c = __dadd_rn(c, e);
}

// Block-level reduction of (sum, compensation) pairs; product f*area is
// itself split exactly with fma.
__global__ void __launch_bounds__(256)
area_partial(const double *__restrict__ f, const double *__restrict__ a, int64_t n,
             double2 *__restrict__ part) {
  double s = 0.0, c = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double p = __dmul_rn(f[i], a[i]);
    const double pe = fma(f[i], a[i], -p);  // exact low part of the product
    acc_pair(s, c, p);
    c = __dadd_rn(c, pe);
  }
  __shared__ double ss[256], cs[256];
  ss[threadIdx.x] = s;
  cs[threadIdx.x] = c;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      double s2, e;
      two_sum(ss[threadIdx.x], ss[threadIdx.x + w], s2, e);
      ss[threadIdx.x] = s2;
      cs[threadIdx.x] = __dadd_rn(__dadd_rn(cs[threadIdx.x], cs[threadIdx.x + w]), e);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = make_double2(ss[0], cs[0]);
}

__global__ void area_final(const double2 *__restrict__ part, int np, double *out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double s = 0.0, c = 0.0;
  for (int i = 0; i < np; ++i) {
    acc_pair(s, c, part[i].x);
    c = __dadd_rn(c, part[i].y);
  }
  out[0] = __dadd_rn(s, c);
}

}  // namespace remap
}  // namespace dccm

using namespace dccm;

// ================================================================ C ABI
extern "C" int dccm_j99_generate(const double *x_LonS, int nxs, const double *y_LatS, int nys,
                                 const double *x_LonD, int nxd, const double *y_LatD, int nyd,
                                 const double *x_LonIntWtS, const double *y_LatIntWtS,
                                 const double *x_LonIntWtD, const double *y_LatIntWtD,
                                 int accuracy_order, int weight_mode, const uint8_t *dst_mask,
                                 dccm_remap_table **table) {
  DCCM_NVTX_FUNC();
  (void)x_LonIntWtS;
  (void)x_LonIntWtD;
  if (!table || !x_LonS || !y_LatS || !x_LonD || !y_LatD || !y_LatIntWtS || !y_LatIntWtD)
    return DCCM_ERR_INVALID_ARG;
  *table = nullptr;
  if (nxs < 1 || nys < 1 || nxd < 1 || nyd < 1) return DCCM_ERR_SHAPE;
  if (accuracy_order < 1 || accuracy_order > 2) return DCCM_ERR_INVALID_ARG;
  if (weight_mode != DCCM_J99_REF && weight_mode != DCCM_J99_CONSERVE) return DCCM_ERR_INVALID_ARG;
  if (weight_mode == DCCM_J99_CONSERVE && accuracy_order != 1) return DCCM_ERR_UNSUPPORTED;
  dccm_remap_table *t = new (std::nothrow) dccm_remap_table();
  if (!t) return DCCM_ERR_NOMEM;
  int st = remap::generate(x_LonS, nxs, y_LatS, nys, x_LonD, nxd, y_LatD, nyd, y_LatIntWtS,
                           y_LatIntWtD, accuracy_order, weight_mode, dst_mask, t);
  if (st != DCCM_OK) {
    delete t;
    return st;
  }
  *table = t;
  return DCCM_OK;
}

extern "C" int dccm_remap_table_size(const dccm_remap_table *t, int64_t *nrow) {
  if (!t || !nrow) return DCCM_ERR_INVALID_ARG;
  *nrow = (int64_t)t->w.size();
  return DCCM_OK;
}

extern "C" int dccm_remap_table_rows(const dccm_remap_table *t, int32_t *iD, int32_t *jD,
                                     int32_t *iS, int32_t *jS, double *w) {
  DCCM_NVTX_FUNC();
  if (!t) return DCCM_ERR_INVALID_ARG;
  const size_t n = t->w.size();
  if (n == 0) return DCCM_OK;
  if (!iD || !jD || !iS || !jS || !w) return DCCM_ERR_INVALID_ARG;
  memcpy(iD, t->iD.data(), n * 4);
  memcpy(jD, t->jD.data(), n * 4);
  memcpy(iS, t->iS.data(), n * 4);
  memcpy(jS, t->jS.data(), n * 4);
  memcpy(w, t->w.data(), n * 8);
  return DCCM_OK;
}

extern "C" int dccm_remap_table_write(const dccm_remap_table *t, const char *path) {
  DCCM_NVTX_FUNC();
  if (!t || !path) return DCCM_ERR_INVALID_ARG;
  FILE *fp = fopen(path, "w");
  if (!fp) return DCCM_ERR_IO;
  for (size_t k = 0; k < t->w.size(); ++k)
    if (fprintf(fp, "%12d%12d%12d%12d  %.17E\n", t->iD[k], t->jD[k], t->iS[k], t->jS[k],
                t->w[k]) < 0) {
      fclose(fp);
      return DCCM_ERR_IO;
    }
  return fclose(fp) == 0 ? DCCM_OK : DCCM_ERR_IO;
}

// Parses one list-directed record "iD jD iS jS w" (commas or blanks; a
// Fortran D exponent is accepted).
static bool parse_row(char *line, int32_t v[4], double *w) {
  for (char *c = line; *c; ++c)
    if (*c == ',') *c = ' ';
    else if (*c == 'D' || *c == 'd') *c = 'E';
  char *p = line, *end = nullptr;
  for (int k = 0; k < 4; ++k) {
    long x = strtol(p, &end, 10);
    if (end == p) return false;
    v[k] = (int32_t)x;
    p = end;
  }
  *w = strtod(p, &end);
  return end != p;
}

extern "C" int dccm_remap_table_read(const char *path, dccm_remap_table **table) {
  DCCM_NVTX_FUNC();
  if (!path || !table) return DCCM_ERR_INVALID_ARG;
  *table = nullptr;
  FILE *fp = fopen(path, "r");
  if (!fp) return DCCM_ERR_IO;
  dccm_remap_table *t = new (std::nothrow) dccm_remap_table();
  if (!t) {
    fclose(fp);
    return DCCM_ERR_NOMEM;
  }
  char buf[512];
  while (fgets(buf, sizeof buf, fp)) {
    bool blank = true;
    for (char *c = buf; *c; ++c)
      if (*c != ' ' && *c != '\t' && *c != '\n' && *c != '\r') blank = false;
    if (blank) continue;
    int32_t v[4];
    double w;
    if (!parse_row(buf, v, &w)) {
      fclose(fp);
      delete t;
      return DCCM_ERR_IO;
    }
    t->iD.push_back(v[0]); t->jD.push_back(v[1]); t->iS.push_back(v[2]); t->jS.push_back(v[3]);
    t->w.push_back(w);
  }
  fclose(fp);
  *table = t;
  return DCCM_OK;
}

extern "C" int dccm_remap_table_index(const dccm_remap_table *t, int GNXS, int GNXR,
                                      int32_t *send_index, int32_t *recv_index, double *coef) {
  DCCM_NVTX_FUNC();
  if (!t) return DCCM_ERR_INVALID_ARG;
  const size_t n = t->w.size();
  if (n == 0) return DCCM_OK;
  if (!send_index || !recv_index || !coef) return DCCM_ERR_INVALID_ARG;
  for (size_t k = 0; k < n; ++k) {
    recv_index[k] = t->iD[k] + GNXR * (t->jD[k] - 1);
    send_index[k] = t->iS[k] + GNXS * (t->jS[k] - 1);
    coef[k] = t->w[k];
  }
  return DCCM_OK;
}

extern "C" int dccm_remap_table_destroy(dccm_remap_table *t) {
  DCCM_NVTX_FUNC();
  delete t;
  return DCCM_OK;
}

extern "C" int dccm_remap_plan_create(int64_t n_send, int64_t n_recv, int64_t nop,
                                      const int32_t *send_index, const int32_t *recv_index,
                                      const double *coef, dccm_remap_plan **plan) {
  DCCM_NVTX_FUNC();
  if (!plan) return DCCM_ERR_INVALID_ARG;
  *plan = nullptr;
  if (n_send < 0 || n_recv < 0 || nop < 0) return DCCM_ERR_INVALID_ARG;
  if (nop > 0 && (!send_index || !recv_index || !coef)) return DCCM_ERR_INVALID_ARG;
  for (int64_t k = 0; k < nop; ++k)
    if (send_index[k] < 1 || send_index[k] > n_send || recv_index[k] < 1 ||
        recv_index[k] > n_recv)
      return DCCM_ERR_INDEX_RANGE;
  if (n_recv >= (1LL << 31) - 32) return DCCM_ERR_UNSUPPORTED;
  // Stable counting sort by destination: per-row order = table order.
  std::vector<int64_t> rowptr(n_recv + 1, 0);
  for (int64_t k = 0; k < nop; ++k) rowptr[recv_index[k]]++;
  for (int64_t r = 0; r < n_recv; ++r) rowptr[r + 1] += rowptr[r];
  // Row order of the slices: by length within windows of 256 rows (stable).
  constexpr int64_t WIN = 256;
  std::vector<int> order((size_t)n_recv);
  for (int64_t r = 0; r < n_recv; ++r) order[(size_t)r] = (int)r;
  for (int64_t w0 = 0; w0 < n_recv; w0 += WIN)
    std::stable_sort(order.begin() + w0, order.begin() + std::min<int64_t>(n_recv, w0 + WIN), [&](int a, int b) {
      return rowptr[a + 1] - rowptr[a] < rowptr[b + 1] - rowptr[b];
    });
  // Sliced ELL: slice q holds rows order[32 q .. 32 q + 31], width = its longest row.
  const int64_t nslice = (n_recv + 31) / 32;
  std::vector<int2> slices((size_t)nslice);
  std::vector<int> rows((size_t)nslice * 32, -1);
  std::vector<int64_t> pos((size_t)n_recv);  // slice position of each row
  int64_t nrec = 0;
  for (int64_t q = 0; q < nslice; ++q) {
    int64_t wmax = 0;
    for (int64_t i = q * 32; i < std::min<int64_t>(n_recv, q * 32 + 32); ++i) {
      const int r = order[(size_t)i];
      wmax = std::max<int64_t>(wmax, rowptr[r + 1] - rowptr[r]);
      rows[(size_t)i] = r;
      pos[(size_t)r] = i;
    }
    if (nrec / 32 > 0x7FFFFFFF || wmax > 0x7FFFFFFF) return DCCM_ERR_UNSUPPORTED;
    slices[(size_t)q] = make_int2((int)(nrec / 32), (int)wmax);
    nrec += 32 * wmax;
  }
  const long long pad = -1;
  double padbits;
  memcpy(&padbits, &pad, sizeof pad);
  std::vector<double2> ent((size_t)nrec, make_double2(0.0, padbits));
  std::vector<int64_t> fill(rowptr.begin(), rowptr.end() - 1);
  for (int64_t k = 0; k < nop; ++k) {
    const int64_t r = recv_index[k] - 1;
    const long long col = (long long)(send_index[k] - 1);
    double colbits;
    memcpy(&colbits, &col, sizeof col);
    const int64_t kk = fill[r]++ - rowptr[r];  // position of the entry within its row
    const int64_t i = pos[(size_t)r];
    ent[(size_t)((int64_t)slices[(size_t)(i / 32)].x * 32 + kk * 32 + i % 32)] = make_double2(coef[k], colbits);
  }
  dccm_remap_plan *p = new (std::nothrow) dccm_remap_plan();
  if (!p) return DCCM_ERR_NOMEM;
  p->n_send = n_send;
  p->n_recv = n_recv;
  p->nnz = nop;
  p->nslice = nslice;
  p->nrec = nrec;
  cudaError_t e = cudaSuccess;
  if (nslice > 0) e = cudaMalloc(&p->d_slices, nslice * sizeof(int2));
  if (e == cudaSuccess && nslice > 0) e = cudaMalloc(&p->d_rows, nslice * 32 * sizeof(int));
  if (e == cudaSuccess && nrec > 0) e = cudaMalloc(&p->d_ent, nrec * sizeof(double2));
  if (e == cudaSuccess && nslice > 0)
    e = cudaMemcpy(p->d_slices, slices.data(), nslice * sizeof(int2), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && nslice > 0)
    e = cudaMemcpy(p->d_rows, rows.data(), nslice * 32 * sizeof(int), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && nrec > 0)
    e = cudaMemcpy(p->d_ent, ent.data(), nrec * sizeof(double2), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    set_cuda_error(e);
    dccm_remap_plan_destroy(p);
    return DCCM_ERR_CUDA;
  }
  *plan = p;
  return DCCM_OK;
}

extern "C" int dccm_remap_plan_destroy(dccm_remap_plan *p) {
  DCCM_NVTX_FUNC();
  if (!p) return DCCM_OK;
  if (p->d_slices) cudaFree(p->d_slices);
  if (p->d_rows) cudaFree(p->d_rows);
  if (p->d_ent) cudaFree(p->d_ent);
  p->stage.release();
  if (p->stream) cudaStreamDestroy(p->stream);
  delete p;
  return DCCM_OK;
}

extern "C" int dccm_remap_plan_info(const dccm_remap_plan *p, int64_t *nnz, int64_t *ns,
                                    int64_t *nr) {
  if (!p) return DCCM_ERR_INVALID_ARG;
  if (nnz) *nnz = p->nnz;
  if (ns) *ns = p->n_send;
  if (nr) *nr = p->n_recv;
  return DCCM_OK;
}

extern "C" int dccm_remap_apply_dev(dccm_remap_plan *p, const double *src, int64_t ld_src,
                                    double *dst, int64_t ld_dst, int nfields, void *stream) {
  DCCM_NVTX_FUNC();
  if (!p || (nfields > 0 && (!src || !dst)) || nfields < 0) return DCCM_ERR_INVALID_ARG;
  if (nfields > 1 && (ld_src < p->n_send || ld_dst < p->n_recv)) return DCCM_ERR_SHAPE;
  return remap::apply(p, src, ld_src, dst, ld_dst, nfields, as_stream(stream));
}

extern "C" int dccm_interpolate_data(dccm_remap_plan *p, int64_t sn1, int64_t sn2,
                                     const double *send_data, int64_t rn1, int64_t rn2,
                                     double *recv_data, int num_of_data) {
  DCCM_NVTX_FUNC();
  if (!p || !send_data || !recv_data || num_of_data < 0) return DCCM_ERR_INVALID_ARG;
  if (sn1 < p->n_send || rn1 < p->n_recv || num_of_data > sn2 || num_of_data > rn2)
    return DCCM_ERR_SHAPE;
  // recv_data(:,:) = 0 (:293): every column, including those past num_of_data.
  if (num_of_data < rn2 || rn1 > p->n_recv) memset(recv_data, 0, sizeof(double) * rn1 * rn2);
  if (num_of_data == 0) return DCCM_OK;
  if (!p->stream) DCCM_CUDA(cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking));
  const size_t sbytes = sizeof(double) * (size_t)sn1 * num_of_data;
  const size_t rbytes = sizeof(double) * (size_t)rn1 * num_of_data;
  DCCM_TRY(p->stage.ensure(sbytes + rbytes));
  double *ds = (double *)p->stage.ptr;
  double *dr = ds + (size_t)sn1 * num_of_data;
  DCCM_CUDA(cudaMemcpyAsync(ds, send_data, sbytes, cudaMemcpyHostToDevice, p->stream));
  if (rn1 > p->n_recv) DCCM_CUDA(cudaMemsetAsync(dr, 0, rbytes, p->stream));
  DCCM_TRY(remap::apply(p, ds, sn1, dr, rn1, num_of_data, p->stream));
  DCCM_CUDA(cudaMemcpyAsync(recv_data, dr, rbytes, cudaMemcpyDeviceToHost, p->stream));
  DCCM_CUDA(cudaStreamSynchronize(p->stream));
  return DCCM_OK;
}

extern "C" int dccm_area_integral_dev(const double *f, const double *area, int64_t n,
                                      double *result, void *stream) {
  DCCM_NVTX_FUNC();
  if (!f || !area || !result || n < 0) return DCCM_ERR_INVALID_ARG;
  cudaStream_t s = as_stream(stream);
  const int threads = 256;
  int np = (int)std::min<int64_t>((n + threads - 1) / threads, (int64_t)sm_count() * 4);
  if (np < 1) np = 1;
  double2 *part;
  double *out;
  DCCM_CUDA(cudaMallocAsync((void **)&part, np * sizeof(double2) + sizeof(double), s));
  out = (double *)(part + np);
  remap::area_partial<<<np, threads, 0, s>>>(f, area, n, part);
  remap::area_final<<<1, 32, 0, s>>>(part, np, out);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(result, out, sizeof(double), cudaMemcpyDeviceToHost, s);
  cudaFreeAsync(part, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    set_cuda_error(e);
    return DCCM_ERR_CUDA;
  }
  return DCCM_OK;
}
