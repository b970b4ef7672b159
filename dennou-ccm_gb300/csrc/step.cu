// The fused coupling step: one CUDA graph per step.
//
// One step of the coupled model's data-parallel hot path on one GPU, as the
// reference runs it across its MPMD components each coupling cycle
// (driver/dccm_atm_driver.f90 -> atm_run, driver/dccm_sfc_driver.f90 ->
// sfc_run): the atmosphere's inverse and forward spectral transforms of all
// field-levels (atm/dcpam_main_mod.f90:2173-2180), the remap of the surface
// fields onto the exchange grid (interpolate_data, called from jcup_get_data
// at sfc/dccm_sfc_mod.f90:865-881) and the bulk flux on that grid
// (sfc/dccm_sfc_mod.f90:886-897).  The MPI exchange of the reference is
// replaced by device buffers shared between graph nodes.
//
// The graph has two branches that run concurrently: spectral transforms
// (inverse then forward), and remap then flux.  dccm_step_run replays it;
// dccm_step_run_timed launches the same stages one after another on one
// stream with events in between (per-stage device times for roofline
// reports); dccm_step_run_host adds the host<->device copies of a caller
// that holds its data in host memory.
#include <new>

#include "sht_plan.cuh"

struct dccm_sht_plan {
  dccm::sht::Plan P;
};
struct dccm_remap_plan;

namespace dccm {
namespace remap {
int apply(dccm_remap_plan *p, const double *src, int64_t ld_src, double *dst, int64_t ld_dst, int nfields,
          cudaStream_t s);
}
namespace sht {
int inverse(Plan &P, const double *spec, double *grid, int batch, cudaStream_t s);
int forward(Plan &P, const double *grid, double *spec, int batch, cudaStream_t s);
}  // namespace sht
}  // namespace dccm

struct dccm_step {
  dccm_step_desc d;
  dccm_sfc_bulk_flux_args flux;
  dccm_sfc_grid fgrid;
  double sig1[2];
  cudaStream_t s0 = nullptr, s1 = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t ev[8] = {};
};

using namespace dccm;

static int stage_sht_inv(dccm_step *st, cudaStream_t s) {
  if (!st->d.sht || st->d.nfl == 0) return DCCM_OK;
  return sht::inverse(st->d.sht->P, st->d.spec_in, st->d.grid, st->d.nfl, s);
}
static int stage_sht_fwd(dccm_step *st, cudaStream_t s) {
  if (!st->d.sht || st->d.nfl == 0) return DCCM_OK;
  return sht::forward(st->d.sht->P, st->d.grid, st->d.spec_out, st->d.nfl, s);
}
static int stage_remap(dccm_step *st, cudaStream_t s) {
  if (!st->d.remap || st->d.nfields == 0) return DCCM_OK;
  return remap::apply(st->d.remap, st->d.remap_src, st->d.ld_src, st->d.remap_dst, st->d.ld_dst,
                      st->d.nfields, s);
}
extern "C" int dccm_sfc_bulk_flux_get_dev(const dccm_sfc_bulk_flux_args *, const dccm_sfc_grid *, void *);
static int stage_flux(dccm_step *st, cudaStream_t s) {
  if (!st->d.flux) return DCCM_OK;
  return dccm_sfc_bulk_flux_get_dev(&st->flux, &st->fgrid, (void *)s);
}

static int record(dccm_step *st) {
  DCCM_CUDA(cudaStreamBeginCapture(st->s0, cudaStreamCaptureModeThreadLocal));
  int rc = DCCM_OK;
  cudaError_t e = cudaEventRecord(st->fork, st->s0);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(st->s1, st->fork, 0);
  if (e != cudaSuccess) rc = DCCM_ERR_CUDA;
  if (rc == DCCM_OK) rc = stage_sht_inv(st, st->s0);
  if (rc == DCCM_OK) rc = stage_sht_fwd(st, st->s0);
  if (rc == DCCM_OK) rc = stage_remap(st, st->s1);
  if (rc == DCCM_OK) rc = stage_flux(st, st->s1);
  if (rc == DCCM_OK) {
    e = cudaEventRecord(st->join, st->s1);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(st->s0, st->join, 0);
    if (e != cudaSuccess) rc = DCCM_ERR_CUDA;
  }
  cudaGraph_t g = nullptr;
  cudaError_t e2 = cudaStreamEndCapture(st->s0, &g);
  if (rc != DCCM_OK) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e2 != cudaSuccess) {
    set_cuda_error(e2);
    return DCCM_ERR_CUDA;
  }
  st->graph = g;
  DCCM_CUDA(cudaGraphInstantiate(&st->exec, g, 0));
  return DCCM_OK;
}

extern "C" int dccm_step_create(const dccm_step_desc *d, dccm_step **out) {
  if (!d || !out) return DCCM_ERR_INVALID_ARG;
  *out = nullptr;
  if (d->nfl < 0 || d->nfields < 0) return DCCM_ERR_INVALID_ARG;
  if (d->sht && d->nfl > d->sht->P.max_batch) return DCCM_ERR_SHAPE;
  if (d->sht && d->nfl > 0 && (!d->spec_in || !d->grid || !d->spec_out)) return DCCM_ERR_INVALID_ARG;
  if (d->remap && d->nfields > 0 && (!d->remap_src || !d->remap_dst)) return DCCM_ERR_INVALID_ARG;
  if (d->flux && (!d->flux_grid || !d->flux->a_Sig1Info)) return DCCM_ERR_INVALID_ARG;
  dccm_step *st = new (std::nothrow) dccm_step();
  if (!st) return DCCM_ERR_NOMEM;
  st->d = *d;
  if (d->flux) {
    st->flux = *d->flux;
    st->fgrid = *d->flux_grid;
    st->sig1[0] = d->flux->a_Sig1Info[0];
    st->sig1[1] = d->flux->a_Sig1Info[1];
    st->flux.a_Sig1Info = st->sig1;
  }
  cudaError_t e = cudaStreamCreateWithFlags(&st->s0, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st->s1, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&st->fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&st->join, cudaEventDisableTiming);
  for (int k = 0; k < 8 && e == cudaSuccess; ++k) e = cudaEventCreate(&st->ev[k]);
  int rc = e == cudaSuccess ? DCCM_OK : DCCM_ERR_CUDA;
  if (e != cudaSuccess) set_cuda_error(e);
  if (rc == DCCM_OK) rc = record(st);
  if (rc != DCCM_OK) {
    dccm_step_destroy(st);
    return rc;
  }
  *out = st;
  return DCCM_OK;
}

extern "C" int dccm_step_destroy(dccm_step *st) {
  if (!st) return DCCM_OK;
  if (st->exec) cudaGraphExecDestroy(st->exec);
  if (st->graph) cudaGraphDestroy(st->graph);
  for (int k = 0; k < 8; ++k)
    if (st->ev[k]) cudaEventDestroy(st->ev[k]);
  if (st->fork) cudaEventDestroy(st->fork);
  if (st->join) cudaEventDestroy(st->join);
  if (st->s0) cudaStreamDestroy(st->s0);
  if (st->s1) cudaStreamDestroy(st->s1);
  delete st;
  return DCCM_OK;
}

extern "C" int dccm_step_run(dccm_step *st, void *stream) {
  if (!st || !st->exec) return DCCM_ERR_INVALID_ARG;
  DCCM_CUDA(cudaGraphLaunch(st->exec, as_stream(stream)));
  return DCCM_OK;
}

extern "C" int dccm_step_run_timed(dccm_step *st, void *stream, float *ms) {
  if (!st || !ms) return DCCM_ERR_INVALID_ARG;
  cudaStream_t s = as_stream(stream);
  int (*stages[4])(dccm_step *, cudaStream_t) = {stage_sht_inv, stage_sht_fwd, stage_remap, stage_flux};
  DCCM_CUDA(cudaEventRecord(st->ev[0], s));
  for (int k = 0; k < 4; ++k) {
    DCCM_TRY(stages[k](st, s));
    DCCM_CUDA(cudaEventRecord(st->ev[k + 1], s));
  }
  DCCM_CUDA(cudaEventSynchronize(st->ev[4]));
  for (int k = 0; k < 4; ++k) DCCM_CUDA(cudaEventElapsedTime(&ms[k], st->ev[k], st->ev[k + 1]));
  return DCCM_OK;
}

extern "C" int dccm_step_run_host(dccm_step *st, void *stream, const dccm_host_copy *h2d, int nh2d,
                                  const dccm_host_copy *d2h, int nd2h) {
  if (!st || (nh2d > 0 && !h2d) || (nd2h > 0 && !d2h) || nh2d < 0 || nd2h < 0) return DCCM_ERR_INVALID_ARG;
  cudaStream_t s = as_stream(stream);
  for (int k = 0; k < nh2d; ++k)
    DCCM_CUDA(cudaMemcpyAsync(h2d[k].dev, h2d[k].host, h2d[k].bytes, cudaMemcpyHostToDevice, s));
  DCCM_CUDA(cudaGraphLaunch(st->exec, s));
  for (int k = 0; k < nd2h; ++k)
    DCCM_CUDA(cudaMemcpyAsync(d2h[k].host, d2h[k].dev, d2h[k].bytes, cudaMemcpyDeviceToHost, s));
  DCCM_CUDA(cudaStreamSynchronize(s));
  return DCCM_OK;
}
