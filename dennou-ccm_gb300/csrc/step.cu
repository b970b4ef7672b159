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
// (inverse then forward; a single plan or an ensemble of truncation groups),
// and the remaps then the flux.  dccm_step_run replays it;
// dccm_step_run_timed launches the same stages one after another on one
// stream with events in between (per-stage device times for roofline
// reports); dccm_step_run_host adds the host<->device copies of a caller
// that holds its data in host memory.
#include <new>
#include <vector>

#include "sht_plan.cuh"

struct dccm_sht_plan {
  dccm::sht::Plan P;
};
struct dccm_remap_plan;

namespace dccm {
namespace remap {
int apply2(dccm_remap_plan *p, const double *src, int64_t ld_src, double *dst, int64_t ld_dst, int nfields,
           int nsub, int64_t ld_dst2, cudaStream_t s);
}
namespace sht {
Plan *ensemble_plan(dccm_sht_ensemble *e, int g);
}  // namespace sht
}  // namespace dccm

struct dccm_step {
  dccm_step_desc d;
  std::vector<const double *> ens_spec_in;
  std::vector<double *> ens_grid, ens_spec_out;
  std::vector<int> ens_nfl;
  std::vector<dccm_step_remap> remaps;
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

// The transforms as four kernel stages: Legendre synthesis, inverse FFT,
// forward FFT, Legendre analysis.  A single plan is group 0 of a list.
struct Groups {
  int n = 0;
  sht::Plan *P[8];
  const double *spec_in[8];
  double *grid[8];
  double *spec_out[8];
  int nfl[8];
};
static Groups groups_of(dccm_step *st) {
  Groups G;
  if (st->d.ens) {
    int ng = 0;
    dccm_sht_ensemble_groups(st->d.ens, &ng);
    for (int g = 0; g < ng && g < 8; ++g) {
      G.P[g] = sht::ensemble_plan(st->d.ens, g);
      G.spec_in[g] = st->ens_spec_in[g];
      G.grid[g] = st->ens_grid[g];
      G.spec_out[g] = st->ens_spec_out[g];
      G.nfl[g] = st->ens_nfl[g];
    }
    G.n = ng;
  } else if (st->d.sht && st->d.nfl > 0) {
    G.P[0] = &st->d.sht->P;
    G.spec_in[0] = st->d.spec_in;
    G.grid[0] = st->d.grid;
    G.spec_out[0] = st->d.spec_out;
    G.nfl[0] = st->d.nfl;
    G.n = 1;
  }
  return G;
}
static bool mixed(const Groups &G) { return G.n > 0 && G.P[0]->precision == DCCM_SHT_MIXED; }

static int stage_leg_inv(dccm_step *st, cudaStream_t s) {
  Groups G = groups_of(st);
  if (G.n == 0) return DCCM_OK;
  if (mixed(G)) {
    void *work[8];
    for (int g = 0; g < G.n; ++g) work[g] = G.P[g]->d_work;
    return sht::legendre_tc_multi(G.P, G.nfl, (const void *const *)G.spec_in, work, G.n, 0, s);
  }
  for (int g = 0; g < G.n; ++g)
    DCCM_TRY(sht::legendre_inv_f64(*G.P[g], G.nfl[g], G.spec_in[g], (double *)G.P[g]->d_work, s));
  return DCCM_OK;
}
static int stage_fft_inv(dccm_step *st, cudaStream_t s) {
  Groups G = groups_of(st);
  if (G.n == 0) return DCCM_OK;
  if (mixed(G)) {
    const void *work[8];
    for (int g = 0; g < G.n; ++g) work[g] = G.P[g]->d_work;
    return sht::fft_multi(G.P, G.nfl, work, (void *const *)G.grid, G.n, false, s);
  }
  for (int g = 0; g < G.n; ++g) DCCM_TRY(sht::fft_inverse(*G.P[g], G.nfl[g], false, G.P[g]->d_work, G.grid[g], s));
  return DCCM_OK;
}
static int stage_fft_fwd(dccm_step *st, cudaStream_t s) {
  Groups G = groups_of(st);
  if (G.n == 0) return DCCM_OK;
  if (mixed(G)) {
    void *work[8];
    for (int g = 0; g < G.n; ++g) work[g] = G.P[g]->d_work;
    return sht::fft_multi(G.P, G.nfl, (const void *const *)G.grid, work, G.n, true, s);
  }
  for (int g = 0; g < G.n; ++g) DCCM_TRY(sht::fft_forward(*G.P[g], G.nfl[g], false, G.grid[g], G.P[g]->d_work, s));
  return DCCM_OK;
}
static int stage_leg_fwd(dccm_step *st, cudaStream_t s) {
  Groups G = groups_of(st);
  if (G.n == 0) return DCCM_OK;
  if (mixed(G)) {
    const void *work[8];
    for (int g = 0; g < G.n; ++g) work[g] = G.P[g]->d_work;
    return sht::legendre_tc_multi(G.P, G.nfl, work, (void *const *)G.spec_out, G.n, 1, s);
  }
  for (int g = 0; g < G.n; ++g)
    DCCM_TRY(sht::legendre_fwd_f64(*G.P[g], G.nfl[g], (const double *)G.P[g]->d_work, G.spec_out[g], s));
  return DCCM_OK;
}
static int stage_sht_inv(dccm_step *st, cudaStream_t s) {
  DCCM_TRY(stage_leg_inv(st, s));
  return stage_fft_inv(st, s);
}
static int stage_sht_fwd(dccm_step *st, cudaStream_t s) {
  DCCM_TRY(stage_fft_fwd(st, s));
  return stage_leg_fwd(st, s);
}
static int stage_remap(dccm_step *st, cudaStream_t s) {
  for (const dccm_step_remap &r : st->remaps)
    if (r.plan && r.nfields > 0)
      DCCM_TRY(remap::apply2(r.plan, r.src, r.ld_src, r.dst, r.ld_dst, r.nfields, r.nsub, r.ld_dst2, s));
  return DCCM_OK;
}
extern "C" int dccm_sfc_bulk_flux_get_dev(const dccm_sfc_bulk_flux_args *, const dccm_sfc_grid *, void *);
static int stage_flux(dccm_step *st, cudaStream_t s) {
  if (!st->d.flux) return DCCM_OK;
  return dccm_sfc_bulk_flux_get_dev(&st->flux, &st->fgrid, (void *)s);
}

static int record(dccm_step *st) {
  // One untimed pass outside capture sets every kernel's attributes.
  DCCM_TRY(stage_sht_inv(st, st->s0));
  DCCM_TRY(stage_sht_fwd(st, st->s0));
  DCCM_TRY(stage_remap(st, st->s0));
  DCCM_TRY(stage_flux(st, st->s0));
  DCCM_CUDA(cudaStreamSynchronize(st->s0));
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
  if (d->nfl < 0 || d->nremap < 0 || (d->nremap > 0 && !d->remaps)) return DCCM_ERR_INVALID_ARG;
  if (d->sht && d->nfl > d->sht->P.max_batch) return DCCM_ERR_SHAPE;
  if (d->sht && d->nfl > 0 && (!d->spec_in || !d->grid || !d->spec_out)) return DCCM_ERR_INVALID_ARG;
  if (d->ens && (!d->ens_spec_in || !d->ens_grid || !d->ens_spec_out || !d->ens_nfl)) return DCCM_ERR_INVALID_ARG;
  for (int k = 0; k < d->nremap; ++k)
    if (d->remaps[k].plan && d->remaps[k].nfields > 0 && (!d->remaps[k].src || !d->remaps[k].dst))
      return DCCM_ERR_INVALID_ARG;
  if (d->flux && (!d->flux_grid || !d->flux->a_Sig1Info)) return DCCM_ERR_INVALID_ARG;
  dccm_step *st = new (std::nothrow) dccm_step();
  if (!st) return DCCM_ERR_NOMEM;
  st->d = *d;
  if (d->ens) {
    int ng = 0;
    DCCM_TRY(dccm_sht_ensemble_groups(d->ens, &ng));
    st->ens_spec_in.assign(d->ens_spec_in, d->ens_spec_in + ng);
    st->ens_grid.assign(d->ens_grid, d->ens_grid + ng);
    st->ens_spec_out.assign(d->ens_spec_out, d->ens_spec_out + ng);
    st->ens_nfl.assign(d->ens_nfl, d->ens_nfl + ng);
  }
  st->remaps.assign(d->remaps, d->remaps + d->nremap);
  st->d.remaps = nullptr;
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
  int (*stages[6])(dccm_step *, cudaStream_t) = {stage_leg_inv, stage_fft_inv, stage_fft_fwd,
                                                  stage_leg_fwd, stage_remap,   stage_flux};
  DCCM_CUDA(cudaEventRecord(st->ev[0], s));
  for (int k = 0; k < 6; ++k) {
    DCCM_TRY(stages[k](st, s));
    DCCM_CUDA(cudaEventRecord(st->ev[k + 1], s));
  }
  DCCM_CUDA(cudaEventSynchronize(st->ev[6]));
  for (int k = 0; k < 6; ++k) DCCM_CUDA(cudaEventElapsedTime(&ms[k], st->ev[k], st->ev[k + 1]));
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

// ------------------------------------------------------------- autotuning
// Launch-shape knobs (common.cuh, Tunables) chosen per step by timing the
// stage each one affects, candidates one knob at a time, with the other
// knobs at their current values; the winners are applied and the step's
// graph is recorded again.  A cache file keeps the choice per step shape
// and GPU, one JSON object per line.
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <string>

static std::string step_key(dccm_step *st) {
  cudaDeviceProp prop;
  int dev = 0;
  cudaGetDevice(&dev);
  cudaGetDeviceProperties(&prop, dev);
  Groups G = groups_of(st);
  char buf[256];
  std::string k = std::string(prop.name) + "/" + std::to_string(prop.multiProcessorCount);
  for (int g = 0; g < G.n; ++g) {
    snprintf(buf, sizeof buf, "|T%d:%dx%d:b%d:p%d", G.P[g]->N, G.P[g]->I, G.P[g]->J, G.nfl[g], G.P[g]->precision);
    k += buf;
  }
  for (const dccm_step_remap &r : st->remaps) {
    snprintf(buf, sizeof buf, "|r%d", r.nfields);
    k += buf;
  }
  if (st->d.flux) {
    snprintf(buf, sizeof buf, "|f%dx%d", st->fgrid.IE - st->fgrid.IS + 1, st->fgrid.JE - st->fgrid.JS + 1);
    k += buf;
  }
  return k;
}

static bool cache_lookup(const char *path, const std::string &key, Tunables &t) {
  if (!path) return false;
  FILE *fp = fopen(path, "r");
  if (!fp) return false;
  char line[2048];
  bool found = false;
  const std::string pat = "\"key\": \"" + key + "\"";
  while (fgets(line, sizeof line, fp)) {
    if (!strstr(line, pat.c_str())) continue;
    Tunables v;
    const char *p;
    if ((p = strstr(line, "\"tc_ctas\": "))) v.tc_ctas = atoi(p + 11);
    if ((p = strstr(line, "\"fft_bb\": "))) v.fft_bb = atoi(p + 10);
    if ((p = strstr(line, "\"flux_threads\": "))) v.flux_threads = atoi(p + 16);
    if ((p = strstr(line, "\"remap_threads\": "))) v.remap_threads = atoi(p + 17);
    t = v;
    found = true;
  }
  fclose(fp);
  return found;
}

static void cache_store(const char *path, const std::string &key, const Tunables &t, const float *ms) {
  if (!path) return;
  FILE *fp = fopen(path, "a");
  if (!fp) return;
  fprintf(fp,
          "{\"key\": \"%s\", \"tc_ctas\": %d, \"fft_bb\": %d, \"flux_threads\": %d, \"remap_threads\": %d, "
          "\"stage_ms\": [%.4f, %.4f, %.4f, %.4f, %.4f, %.4f]}\n",
          key.c_str(), t.tc_ctas, t.fft_bb, t.flux_threads, t.remap_threads, ms[0], ms[1], ms[2], ms[3], ms[4],
          ms[5]);
  fclose(fp);
}

// Median over reps of the device time of the stages in [k0, k1).
static int time_stages(dccm_step *st, cudaStream_t s, int k0, int k1, int reps, float *out) {
  std::vector<float> v;
  float ms[6];
  for (int r = 0; r < reps; ++r) {
    DCCM_TRY(dccm_step_run_timed(st, s, ms));
    float sum = 0.f;
    for (int k = k0; k < k1; ++k) sum += ms[k];
    v.push_back(sum);
  }
  std::sort(v.begin(), v.end());
  *out = v[v.size() / 2];
  return DCCM_OK;
}

extern "C" int dccm_step_autotune(dccm_step *st, const char *cache_path, int *chosen) {
  if (!st) return DCCM_ERR_INVALID_ARG;
  Tunables &T = tunables();
  const Tunables saved = T;
  const std::string key = step_key(st);
  Tunables best = T;
  float ms[6] = {0, 0, 0, 0, 0, 0};
  if (!cache_lookup(cache_path, key, best)) {
    cudaStream_t s = st->s0;
    const int sms = sm_count();
    struct Knob {
      int *field;
      std::vector<int> cand;
      int k0, k1;
    } knobs[] = {
        {&T.tc_ctas, {sms, sms * 3 / 4, sms / 2, sms / 4}, 0, 4},
        {&T.fft_bb, {8, 4, 2, 1}, 1, 3},
        {&T.flux_threads, {64, 128, 256}, 5, 6},
        {&T.remap_threads, {128, 256}, 4, 5},
    };
    for (Knob &kb : knobs) {
      int bestv = *kb.field;
      float bt = 1e30f;
      for (int c : kb.cand) {
        *kb.field = c;
        float t;
        const int rc = time_stages(st, s, kb.k0, kb.k1, 7, &t);
        if (rc != DCCM_OK) {
          T = saved;
          return rc;
        }
        if (t < bt) {
          bt = t;
          bestv = c;
        }
      }
      *kb.field = bestv;
    }
    best = T;
    DCCM_TRY(dccm_step_run_timed(st, s, ms));
    cache_store(cache_path, key, best, ms);
  }
  T = best;
  // Record the graph again with the chosen launch shapes.
  if (st->exec) cudaGraphExecDestroy(st->exec);
  if (st->graph) cudaGraphDestroy(st->graph);
  st->exec = nullptr;
  st->graph = nullptr;
  const int rc = record(st);
  if (chosen) {
    chosen[0] = best.tc_ctas;
    chosen[1] = best.fft_bb;
    chosen[2] = best.flux_threads;
    chosen[3] = best.remap_threads;
  }
  return rc;
}

extern "C" int dccm_tune_set(const char *knob, int value) {
  if (!knob || value < 0) return DCCM_ERR_INVALID_ARG;
  Tunables &T = tunables();
  if (!strcmp(knob, "tc_ctas")) T.tc_ctas = value;
  else if (!strcmp(knob, "fft_bb")) T.fft_bb = value;
  else if (!strcmp(knob, "flux_threads")) T.flux_threads = value;
  else if (!strcmp(knob, "remap_threads")) T.remap_threads = value;
  else return DCCM_ERR_INVALID_ARG;
  return DCCM_OK;
}

extern "C" int dccm_tune_get(const char *knob, int *value) {
  if (!knob || !value) return DCCM_ERR_INVALID_ARG;
  const Tunables &T = tunables();
  if (!strcmp(knob, "tc_ctas")) *value = T.tc_ctas;
  else if (!strcmp(knob, "fft_bb")) *value = T.fft_bb;
  else if (!strcmp(knob, "flux_threads")) *value = T.flux_threads;
  else if (!strcmp(knob, "remap_threads")) *value = T.remap_threads;
  else return DCCM_ERR_INVALID_ARG;
  return DCCM_OK;
}
