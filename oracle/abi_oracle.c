/*
 * abi_oracle.c -- the include/eprem_gpu.h entry points that
 * eprem_gb300/host/eprem_dropin.c calls, computed by the CPU restatement
 * (eprem_oracle.c).  TEST INFRASTRUCTURE ONLY: it is linked into one test
 * binary, oracle/_ref/eprem_oracle_dropin (the reference's unchanged driver
 * src/eprem.c + the drop-in + this file), never into libeprem_gpu.so, and no
 * product path loads it.
 *
 * What it proves: run over the reference's testsuite configurations, that
 * binary must reproduce the testsuite's golden digests.  That pins, on whole
 * runs (grid construction, shell spawning, output, ideal shock), both the
 * restatement and the drop-in's packing of the reference globals into the
 * ABI's arrays -- the packing the GPU build uses unchanged.
 */
#include <float.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "eprem_oracle.h"

struct eprem_gpu_run {
  eprem_dims_t d;
  eprem_params_t p;
  eprem_grids_t g;
  double *f, *nodes;
  eprem_ep_stats_t stats;
  int mas_ready, mas_on;
  eprem_mas_slice_t slot[2];
  orc_mas_t mas;
};

static char abi_err[320] = "";

static int abi_fail(int code, const char *what) {
  snprintf(abi_err, sizeof(abi_err), "%s", what);
  return code;
}

static void stats_reset(eprem_ep_stats_t *s) {
  memset(s, 0, sizeof(*s));
  s->min_tau = DBL_MAX;
}

const char *eprem_gpu_last_error(void) { return abi_err; }

int eprem_gpu_create(const eprem_dims_t *d, const eprem_params_t *p, const eprem_grids_t *g,
                     eprem_gpu_run **out) {
  if (!d || !p || !g || !out) return abi_fail(EPREM_GPU_ERR_ARG, "null argument");
  if (d->precision != EPREM_FP64) return abi_fail(EPREM_GPU_ERR_ARG, "the oracle is FP64 only");
  eprem_gpu_run *r = (eprem_gpu_run *)calloc(1, sizeof(*r));
  r->d = *d;
  r->p = *p;
  r->g = *g;  /* the reference's grid arrays live for the whole process */
  const size_t sn = (size_t)d->num_streams * d->num_nodes;
  r->f = (double *)calloc(sn * d->num_energies * d->num_mu, sizeof(double));
  r->nodes = (double *)calloc(sn * EPREM_NODE_NFIELDS, sizeof(double));
  stats_reset(&r->stats);
  *out = r;
  return EPREM_GPU_OK;
}

int eprem_gpu_upload_f(eprem_gpu_run *r, const double *f) {
  const size_t n = (size_t)r->d.num_streams * r->d.num_nodes * r->d.num_energies * r->d.num_mu;
  memcpy(r->f, f, n * sizeof(double));
  return EPREM_GPU_OK;
}
int eprem_gpu_download_f(eprem_gpu_run *r, double *f) {
  const size_t n = (size_t)r->d.num_streams * r->d.num_nodes * r->d.num_energies * r->d.num_mu;
  memcpy(f, r->f, n * sizeof(double));
  return EPREM_GPU_OK;
}
int eprem_gpu_upload_nodes(eprem_gpu_run *r, const double *nodes, uint64_t mask) {
  const size_t sn = (size_t)r->d.num_streams * r->d.num_nodes;
  for (int k = 0; k < EPREM_NODE_NFIELDS; k++)
    if (mask & EPREM_NODE_MASK(k)) memcpy(r->nodes + k * sn, nodes + k * sn, sn * sizeof(double));
  return EPREM_GPU_OK;
}
int eprem_gpu_download_nodes(eprem_gpu_run *r, double *nodes, uint64_t mask) {
  const size_t sn = (size_t)r->d.num_streams * r->d.num_nodes;
  for (int k = 0; k < EPREM_NODE_NFIELDS; k++)
    if (mask & EPREM_NODE_MASK(k)) memcpy(nodes + k * sn, r->nodes + k * sn, sn * sizeof(double));
  return EPREM_GPU_OK;
}

/* EPREM_ORACLE_THREADS: streams are split across that many POSIX threads
 * (independent when drift and shell diffusion are off); results do not
 * depend on it. */
int eprem_gpu_update_energetic_particles(eprem_gpu_run *r, double t_global) {
  (void)t_global;
  char err[256] = "";
  const char *env = getenv("EPREM_ORACLE_THREADS");
  const int nt = env ? atoi(env) : 1;
  const int rc = orc_update_energetic_particles(&r->d, &r->p, &r->g, r->f, r->nodes, &r->stats,
                                                nt > 0 ? nt : 1, err);
  return rc == EPREM_GPU_OK ? rc : abi_fail(rc, err);
}
int eprem_gpu_read_stats(eprem_gpu_run *r, eprem_ep_stats_t *s) {
  *s = r->stats;
  stats_reset(&r->stats);
  return EPREM_GPU_OK;
}

int eprem_gpu_update_mhd(eprem_gpu_run *r, double t_global) {
  const int rc = r->mas_on ? orc_mas_update_mhd(&r->d, &r->p, r->nodes, &r->mas, t_global)
                           : orc_update_mhd(&r->d, &r->p, r->nodes, t_global);
  return rc == EPREM_GPU_OK ? rc : abi_fail(rc, "updateMhd");
}
int eprem_gpu_move_nodes(eprem_gpu_run *r, double dt) {
  const int rc = orc_move_nodes(&r->d, &r->p, r->nodes, dt);
  return rc == EPREM_GPU_OK ? rc : abi_fail(rc, "moveNodes");
}

int eprem_gpu_set_time_step(eprem_gpu_run *r, double t_del) {
  if (!(t_del > 0.0)) return abi_fail(EPREM_GPU_ERR_ARG, "t_del must be > 0");
  r->p.t_del = t_del;
  return EPREM_GPU_OK;
}

int eprem_gpu_mas_init(eprem_gpu_run *r, const eprem_mas_params_t *mp) {
  r->mas.p = *mp;
  r->mas.slot0 = &r->slot[0];
  r->mas.slot1 = &r->slot[1];
  r->mas_ready = 1;
  r->mas_on = 1;
  return EPREM_GPU_OK;
}
int eprem_gpu_mas_load_slice(eprem_gpu_run *r, int slot, const eprem_mas_slice_t *sl) {
  if (!r->mas_ready || slot < 0 || slot > 1) return abi_fail(EPREM_GPU_ERR_ARG, "MAS slot");
  r->slot[slot] = *sl;  /* the reference keeps its slot arrays until the next read */
  return EPREM_GPU_OK;
}
int eprem_gpu_mas_select(eprem_gpu_run *r, int s0, int s1, double s_cor, double phi_offset) {
  if (!r->mas_ready || s0 < 0 || s0 > 1 || s1 < 0 || s1 > 1)
    return abi_fail(EPREM_GPU_ERR_ARG, "MAS slots");
  r->mas.slot0 = &r->slot[s0];
  r->mas.slot1 = &r->slot[s1];
  r->mas.s_cor = s_cor;
  r->mas.phi_offset = phi_offset;
  return EPREM_GPU_OK;
}
int eprem_gpu_mas_use(eprem_gpu_run *r, int use_mas) {
  if (!r->mas_ready) return abi_fail(EPREM_GPU_ERR_ARG, "MAS not initialised");
  r->mas_on = use_mas != 0;
  return EPREM_GPU_OK;
}
int eprem_gpu_mas_move_nodes(eprem_gpu_run *r, double dt) {
  if (!r->mas_ready) return abi_fail(EPREM_GPU_ERR_ARG, "MAS not initialised");
  const int rc = orc_mas_move_nodes(&r->d, &r->p, r->nodes, &r->mas, dt);
  return rc == EPREM_GPU_OK ? rc : abi_fail(rc, "masMoveNodes");
}
