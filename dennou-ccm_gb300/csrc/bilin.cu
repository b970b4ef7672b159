// Bilinear remap table and the surface exchange grid.
//
// dccm_bilinear_generate replaces gen_gridmapfile_lonlat2lonlat of
// common/grid_mapping_util.f90:32-182 (the non-conservative mapping the
// coupler's GMAPTAG_* tags use; tool/gmapgen/gmapgen_main.f90:100-117).
// The host finds, per destination latitude, the source latitude row
// (get_correspondID_latS :130-150) and the branch, and lays the rows out in
// the reference's order; the GPU evaluates every row, one thread each, with
// the reference's expressions (cal_coef :152-163, cal_coef_axisym :165-174),
// so the weights are the reference's bit for bit.  One place is given a
// meaning: north of the last source latitude on a grid that is not
// axisymmetric, cal_coef reads y_LatS(nys+1) past the end of the array;
// there the rows extrapolate from the last two source latitudes, the mirror
// image of the reference's own south edge (latR <= y_LatS(1) uses rows 1
// and 2 with a negative weight).
//
// dccm_exchange_grid replaces generate_surface_exchage_grid of
// tool/gmapgen/gmapgen_main.f90:336-405 (sort :407-425): the latitude cells
// of the surface exchange grid are the union of the atmosphere's and the
// ocean's (edges from the sin-latitude widths), cells narrower than 1e-12
// in sin(latitude) dropped.  Host arithmetic (a few hundred values).
#include <math.h>

#include <new>
#include <vector>

#include "common.cuh"
#include "remap_table.cuh"
#include "nvtx.cuh"

namespace dccm {
namespace bilin {

enum { GENERAL = 0, AXI_DST = 1, AXI_SRC = 2 };

// Per destination latitude: branch, source row js (or the extrapolation
// base jb), whether the latitude lies outside the source rows, first row.
struct Lat {
  long long row0;
  int js, extp, branch, count;
};

struct Params {
  const double *lonS, *latS, *lonR, *latR;
  int nxs, nys, nxr, nyr;
  double dlon_r, dlon_s;
  const Lat *lat;
  int32_t *iR, *jR, *iS, *jS;
  double *w;
};

__global__ void __launch_bounds__(256) rows_kernel(const Params p) {
  const int jr = blockIdx.y + 1;
  const Lat L = p.lat[jr - 1];
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= L.count) return;
  const long long o = L.row0 + r;
  const int js = L.js, nxs = p.nxs, nys = p.nys;
  int ir, is, jsx;
  double wt;
  if (L.branch == GENERAL) {  // :108-125, four corners per destination cell
    ir = r / 4 + 1;
    const int corner = r % 4;
    is = (int)(p.dlon_r * (ir - 1) / p.dlon_s) + 1;
    const double xc = p.lonR[ir - 1], yc = p.latR[jr - 1];
    const double x1 = p.lonS[is - 1], y1 = p.latS[js - 1];
    const double x3 = p.lonS[is % nxs], y3 = p.latS[js];
    const double a1 = (xc - x1) / (x3 - x1), a2 = 1.0 - a1;
    const double b1 = (yc - y1) / (y3 - y1), b2 = 1.0 - b1;
    const int is2 = is % nxs + 1, js2 = js % nys + 1;
    switch (corner) {
      case 0: wt = a2 * b2; jsx = js; break;
      case 1: wt = a1 * b2; is = is2; jsx = js; break;
      case 2: wt = a1 * b1; is = is2; jsx = js2; break;
      default: wt = a2 * b1; jsx = js2; break;
    }
  } else {
    const double b1 =
        L.extp ? 0.0 : (p.latR[jr - 1] - p.latS[js - 1]) / (p.latS[js] - p.latS[js - 1]);
    const int per = L.extp ? 1 : 2;
    const int k = r / per, part = r % per;
    jsx = part ? js % nys + 1 : js;
    if (L.branch == AXI_DST) {  // :84-95, destination axisymmetric
      ir = 1;
      is = k + 1;
      wt = L.extp ? 1.0 / nxs : (part ? b1 / nxs : (1.0 - b1) / nxs);
    } else {  // :96-106, source axisymmetric
      ir = k + 1;
      is = 1;
      wt = L.extp ? 1.0 : (part ? b1 : 1.0 - b1);
    }
  }
  p.iR[o] = ir;
  p.jR[o] = jr;
  p.iS[o] = is;
  p.jS[o] = jsx;
  p.w[o] = wt;
}

// get_correspondID_latS (:130-150); 0 if neither bound holds (NaN).
static int corresp_lat(double latR, const double *y, int nys, int *extp) {
  for (int j = 1; j <= nys - 1; ++j)
    if (y[j - 1] < latR && latR <= y[j]) {
      *extp = 0;
      return j;
    }
  *extp = 1;
  int id = 0;
  if (latR <= y[0]) id = 1;
  if (latR > y[nys - 1]) id = nys;
  return id;
}

}  // namespace bilin
}  // namespace dccm

using namespace dccm;

extern "C" int dccm_bilinear_generate(const double *x_LonS, int nxs, const double *y_LatS, int nys,
                                      const double *x_LonR, int nxr, const double *y_LatR, int nyr,
                                      const uint8_t *dst_mask, dccm_remap_table **table) {
  DCCM_NVTX_FUNC();
  if (!table || !x_LonS || !y_LatS || !x_LonR || !y_LatR) return DCCM_ERR_INVALID_ARG;
  *table = nullptr;
  if (nxs < 1 || nys < 1 || nxr < 1 || nyr < 1 || nyr > 65535) return DCCM_ERR_SHAPE;
  const int branch = nxr == 1 ? bilin::AXI_DST : (nxs == 1 ? bilin::AXI_SRC : bilin::GENERAL);
  if (branch == bilin::GENERAL && nys < 2) return DCCM_ERR_UNSUPPORTED;
  std::vector<bilin::Lat> lat(nyr);
  long long rows = 0;
  int maxc = 0;
  for (int jr = 1; jr <= nyr; ++jr) {
    bilin::Lat &L = lat[jr - 1];
    L.js = bilin::corresp_lat(y_LatR[jr - 1], y_LatS, nys, &L.extp);
    if (L.js == 0) return DCCM_ERR_SEARCH;
    L.branch = branch;
    if (branch == bilin::GENERAL) {
      if (L.extp && L.js == nys) L.js = nys - 1;  // see the file header
      L.count = 4 * nxr;
    } else {
      const int n = branch == bilin::AXI_DST ? nxs : nxr;
      L.count = L.extp ? n : 2 * n;
    }
    L.row0 = rows;
    rows += L.count;
    maxc = L.count > maxc ? L.count : maxc;
  }
  if (rows >= (1LL << 31)) return DCCM_ERR_UNSUPPORTED;
  dccm_remap_table *t = new (std::nothrow) dccm_remap_table();
  if (!t) return DCCM_ERR_NOMEM;
  // device buffers: grids, per-latitude records, rows
  const size_t gbytes = (size_t)(nxs + nys + nxr + nyr) * sizeof(double);
  const size_t lbytes = (size_t)nyr * sizeof(bilin::Lat);
  const size_t rbytes = (size_t)rows * (4 * sizeof(int32_t) + sizeof(double));
  DevBuf buf;
  int st = buf.ensure(gbytes + lbytes + rbytes + 64);
  if (st != DCCM_OK) {
    delete t;
    return st;
  }
  unsigned char *base = static_cast<unsigned char *>(buf.ptr);
  double *g = reinterpret_cast<double *>(base);
  bilin::Lat *dl = reinterpret_cast<bilin::Lat *>(base + gbytes);
  double *dw = reinterpret_cast<double *>(base + ((gbytes + lbytes + 15) / 16) * 16);
  int32_t *di = reinterpret_cast<int32_t *>(dw + rows);
  bilin::Params p;
  p.lonS = g;
  p.latS = g + nxs;
  p.lonR = g + nxs + nys;
  p.latR = g + nxs + nys + nxr;
  p.nxs = nxs;
  p.nys = nys;
  p.nxr = nxr;
  p.nyr = nyr;
  p.dlon_r = 360.0 / (double)nxr;  // :74-75 (degrees)
  p.dlon_s = 360.0 / (double)nxs;
  p.lat = dl;
  p.w = dw;
  p.iR = di;
  p.jR = di + rows;
  p.iS = di + 2 * rows;
  p.jS = di + 3 * rows;
  cudaError_t e = cudaMemcpy(g, x_LonS, nxs * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(g + nxs, y_LatS, nys * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(g + nxs + nys, x_LonR, nxr * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(g + nxs + nys + nxr, y_LatR, nyr * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dl, lat.data(), lbytes, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && rows > 0) {
    bilin::rows_kernel<<<dim3((unsigned)((maxc + 255) / 256), (unsigned)nyr), 256>>>(p);
    e = cudaGetLastError();
  }
  std::vector<int32_t> iR(rows), jR(rows), iS(rows), jS(rows);
  std::vector<double> w(rows);
  if (e == cudaSuccess && rows > 0) e = cudaMemcpy(w.data(), dw, rows * sizeof(double), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && rows > 0)
    e = cudaMemcpy(iR.data(), p.iR, rows * sizeof(int32_t), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && rows > 0)
    e = cudaMemcpy(jR.data(), p.jR, rows * sizeof(int32_t), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && rows > 0)
    e = cudaMemcpy(iS.data(), p.iS, rows * sizeof(int32_t), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && rows > 0)
    e = cudaMemcpy(jS.data(), p.jS, rows * sizeof(int32_t), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) {
    set_cuda_error(e);
    delete t;
    return DCCM_ERR_CUDA;
  }
  // land mask: drop the rows of masked destination cells (the reference has none)
  for (long long k = 0; k < rows; ++k) {
    if (dst_mask && !dst_mask[(iR[k] - 1) + (long long)nxr * (jR[k] - 1)]) continue;
    t->iD.push_back(iR[k]);
    t->jD.push_back(jR[k]);
    t->iS.push_back(iS[k]);
    t->jS.push_back(jS[k]);
    t->w.push_back(w[k]);
  }
  *table = t;
  return DCCM_OK;
}

extern "C" int dccm_exchange_grid(const double *y_LatA, const double *y_IntWtLatA, int JMA, const double *y_LatO,
                                  const double *y_IntWtLatO, int JMO, double *y_LatX, double *y_IntWtLatX,
                                  int *JMX) {
  DCCM_NVTX_FUNC();
  if (!y_LatA || !y_IntWtLatA || !y_IntWtLatO || !y_LatX || !y_IntWtLatX || !JMX) return DCCM_ERR_INVALID_ARG;
  if (JMA < 1 || JMO < 1) return DCCM_ERR_SHAPE;
  (void)y_LatO;
  if (JMA == JMO) {  // :352-357
    for (int j = 0; j < JMA; ++j) {
      y_LatX[j] = y_LatA[j];
      y_IntWtLatX[j] = y_IntWtLatA[j];
    }
    *JMX = JMA;
    return DCCM_OK;
  }
  const double PI = acos(-1.0);
  const int JMS_ = JMO + JMA - 1;
  std::vector<double> FJA(JMA + 1), FJO(JMO + 1), FJS(JMS_ + 1);
  FJA[0] = -PI / 2.0;  // :361-365
  for (int j = 1; j <= JMA; ++j) FJA[j] = asin(y_IntWtLatA[j - 1] + sin(FJA[j - 1]));
  FJA[JMA] = PI / 2.0;
  FJO[0] = -PI / 2.0;  // :367-371
  for (int j = 1; j <= JMO - 1; ++j) FJO[j] = asin(y_IntWtLatO[j - 1] + sin(FJO[j - 1]));
  FJO[JMO] = PI / 2.0;
  for (int j = 0; j <= JMA - 1; ++j) FJS[j] = FJA[j];  // :373-374
  for (int j = 1; j <= JMO; ++j) FJS[JMA - 1 + j] = FJO[j];
  // sort (:407-425) as the reference does it (an exchange sort; equal keys
  // keep no particular order, which does not change the values)
  const int N = JMS_ + 1;
  for (int i = 0; i < N - 1; ++i)
    for (int j = i + 1; j < N; ++j)
      if (FJS[i] > FJS[j]) {
        const double tmp = FJS[i];
        FJS[i] = FJS[j];
        FJS[j] = tmp;
      }
  int n = 0;  // :380-388
  for (int j = 1; j <= JMS_; ++j) {
    const double intWt = sin(FJS[j]) - sin(FJS[j - 1]);
    if (fabs(intWt) > 1e-12) {
      y_LatX[n] = 0.5 * (FJS[j - 1] + FJS[j]);
      y_IntWtLatX[n] = intWt;
      ++n;
    }
  }
  *JMX = n;
  return DCCM_OK;
}
