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
 *
 * Recording (for tests/golden/make_testsuite_calls.py): with
 * EPREM_ORACLE_RECORD=<dir>, every compute call (updateEnergeticParticles,
 * updateMhd, moveNodes, masMoveNodes, numbered from 0 in call order) appends
 * "<index> <kind> <argument>" to <dir>/calls.txt; with
 * EPREM_ORACLE_RECORD_AT=<i,j,...> as well, the inputs of calls i, j, ...
 * (dimensions, parameters, grids, f, every node field, the MAS slots) are
 * written to <dir>/call_<i>.rec before the call runs, as named arrays:
 * int32 name length, name, int32 type (0 float64, 1 float32, 2 int32, 3 raw
 * bytes), int64 count, values.
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
  int32_t *news; /* shell diffusion: NEWS links, NULL when off */
  double kperxkpar;
  int drift_on;          /* drift: curl formed by updateMhd                  */
  eprem_drift_params_t drift;
  int32_t *drift_news;   /* drift: NEWS links once known                     */
  double *curl;          /* [3][S*N]                                         */
};

static char abi_err[320] = "";

static int abi_fail(int code, const char *what) {
  snprintf(abi_err, sizeof(abi_err), "%s", what);
  return code;
}

/* ---- call recording ---------------------------------------------------- */
enum { REC_EP = 0, REC_MHD = 1, REC_MOVE = 2, REC_MAS_MOVE = 3 };
static long rec_index = 0;

static void rec_put(FILE *fp, const char *name, int type, const void *data, int64_t count) {
  static const int size[4] = {8, 4, 4, 1};
  const int32_t nl = (int32_t)strlen(name), t = type;
  fwrite(&nl, 4, 1, fp);
  fwrite(name, 1, (size_t)nl, fp);
  fwrite(&t, 4, 1, fp);
  fwrite(&count, 8, 1, fp);
  if (count > 0) fwrite(data, (size_t)size[type], (size_t)count, fp);
}

static int rec_wanted(long idx) {
  const char *at = getenv("EPREM_ORACLE_RECORD_AT");
  if (!at) return 0;
  const char *p = at;
  while (*p) {
    char *end;
    const long v = strtol(p, &end, 10);
    if (end == p) break;
    if (v == idx) return 1;
    p = (*end == ',') ? end + 1 : end;
  }
  return 0;
}

static void rec_call(const eprem_gpu_run *r, int kind, double arg) {
  const char *dir = getenv("EPREM_ORACLE_RECORD");
  const long idx = rec_index++;
  if (!dir) return;
  char path[1024];
  snprintf(path, sizeof(path), "%s/calls.txt", dir);
  FILE *fp = fopen(path, "a");
  if (fp) {
    fprintf(fp, "%ld %d %.17g\n", idx, kind, arg);
    fclose(fp);
  }
  if (!rec_wanted(idx)) return;
  snprintf(path, sizeof(path), "%s/call_%ld.rec", dir, idx);
  fp = fopen(path, "wb");
  if (!fp) return;
  const int32_t k = kind, mas_on = r->mas_on;
  const eprem_dims_t *d = &r->d;
  const int64_t E = d->num_energies, M = d->num_mu;
  const int64_t sn = (int64_t)d->num_streams * d->num_nodes;
  rec_put(fp, "kind", 2, &k, 1);
  rec_put(fp, "arg", 0, &arg, 1);
  rec_put(fp, "dims", 3, d, (int64_t)sizeof(*d));
  rec_put(fp, "params", 3, &r->p, (int64_t)sizeof(r->p));
  rec_put(fp, "egrid", 0, r->g.egrid, E);
  rec_put(fp, "vgrid", 0, r->g.vgrid, E);
  rec_put(fp, "vgrid_i", 0, r->g.vgrid_i, E);
  rec_put(fp, "rigidity", 0, r->g.rigidity, E);
  rec_put(fp, "mugrid", 0, r->g.mugrid, M);
  rec_put(fp, "dlnp", 0, &r->g.dlnp, 1);
  rec_put(fp, "dmu", 0, &r->g.dmu, 1);
  if (kind == REC_EP) rec_put(fp, "f", 0, r->f, sn * E * M);
  if (kind == REC_EP && r->news) {
    rec_put(fp, "news", 2, r->news, 4 * (int64_t)d->num_streams);
    rec_put(fp, "kperxkpar", 0, &r->kperxkpar, 1);
  }
  rec_put(fp, "nodes", 0, r->nodes, sn * EPREM_NODE_NFIELDS);
  rec_put(fp, "mas_on", 2, &mas_on, 1);
  if (r->mas_ready) {
    rec_put(fp, "mas_params", 3, &r->mas.p, (int64_t)sizeof(r->mas.p));
    rec_put(fp, "s_cor", 0, &r->mas.s_cor, 1);
    rec_put(fp, "phi_offset", 0, &r->mas.phi_offset, 1);
    const eprem_mas_slice_t *sl[2] = {r->mas.slot0, r->mas.slot1};
    for (int s = 0; s < 2; s++) {
      char nm[64];
      snprintf(nm, sizeof(nm), "slot%d_dims", s);
      rec_put(fp, nm, 2, sl[s]->dims, 3 * EPREM_MAS_NFIELDS);
      for (int fld = 0; fld < EPREM_MAS_NFIELDS; fld++) {
        const int64_t nr = sl[s]->dims[fld][0], nt = sl[s]->dims[fld][1], np = sl[s]->dims[fld][2];
        for (int a = 0; a < 3; a++) {
          snprintf(nm, sizeof(nm), "slot%d_mesh%d_%d", s, fld, a);
          rec_put(fp, nm, 1, sl[s]->mesh[fld][a], sl[s]->dims[fld][a]);
        }
        snprintf(nm, sizeof(nm), "slot%d_data%d", s, fld);
        rec_put(fp, nm, 1, sl[s]->data[fld], nr * nt * np);
      }
    }
  }
  fclose(fp);
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
int eprem_gpu_upload_f_pitched(eprem_gpu_run *r, const double *f, size_t stream_pitch) {
  const size_t per = (size_t)r->d.num_nodes * r->d.num_energies * r->d.num_mu;
  const size_t pitch = stream_pitch ? stream_pitch : per;
  if (pitch < per) return abi_fail(EPREM_GPU_ERR_ARG, "stream_pitch below N*E*M");
  for (int s = 0; s < r->d.num_streams; s++)
    memcpy(r->f + (size_t)s * per, f + (size_t)s * pitch, per * sizeof(double));
  return EPREM_GPU_OK;
}
int eprem_gpu_download_f_pitched(eprem_gpu_run *r, double *f, size_t stream_pitch) {
  const size_t per = (size_t)r->d.num_nodes * r->d.num_energies * r->d.num_mu;
  const size_t pitch = stream_pitch ? stream_pitch : per;
  if (pitch < per) return abi_fail(EPREM_GPU_ERR_ARG, "stream_pitch below N*E*M");
  for (int s = 0; s < r->d.num_streams; s++)
    memcpy(f + (size_t)s * pitch, r->f + (size_t)s * per, per * sizeof(double));
  return EPREM_GPU_OK;
}
/* rippleShellsOut (src/simCore.c:700-735) for f held here */
int eprem_gpu_ripple_f(eprem_gpu_run *r, const double *tmpl, size_t stream_pitch) {
  const size_t em = (size_t)r->d.num_energies * r->d.num_mu;
  const size_t pitch = stream_pitch ? stream_pitch : em;
  const int N = r->d.num_nodes;
  if (pitch < em) return abi_fail(EPREM_GPU_ERR_ARG, "stream_pitch below E*M");
  for (int s = 0; s < r->d.num_streams; s++) {
    double *p = r->f + (size_t)s * N * em;
    memmove(p + em, p, (size_t)(N - 1) * em * sizeof(double));
    memcpy(p, tmpl + (size_t)s * pitch, em * sizeof(double));
  }
  return EPREM_GPU_OK;
}

int eprem_gpu_omni_flux(eprem_gpu_run *r, double *out) {
  if (!r || !out) return abi_fail(EPREM_GPU_ERR_ARG, "null argument");
  orc_omni_flux(&r->d, &r->g, r->f, out);
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
  rec_call(r, REC_EP, t_global);
  char err[256] = "";
  const char *env = getenv("EPREM_ORACLE_THREADS");
  const int nt = env ? atoi(env) : 1;
  const int drift = r->drift_on && r->drift_news;
  int rc;
  if (drift) {
    if (r->news && memcmp(r->news, r->drift_news, 4 * sizeof(int32_t) * r->d.num_streams))
      return abi_fail(EPREM_GPU_ERR_ARG, "shell diffusion and drift need the same links");
    rc = orc_update_energetic_particles_perp(&r->d, &r->p, &r->g, r->f, r->nodes, r->drift_news,
                                             r->news != NULL, r->kperxkpar, &r->drift, r->curl,
                                             &r->stats, nt > 0 ? nt : 1, err);
  } else {
    rc = r->news ? orc_update_energetic_particles_news(&r->d, &r->p, &r->g, r->f, r->nodes,
                                                       r->news, r->kperxkpar, &r->stats,
                                                       nt > 0 ? nt : 1, err)
                 : orc_update_energetic_particles(&r->d, &r->p, &r->g, r->f, r->nodes,
                                                  &r->stats, nt > 0 ? nt : 1, err);
  }
  return rc == EPREM_GPU_OK ? rc : abi_fail(rc, err);
}
void *eprem_gpu_host_alloc(size_t bytes) { return malloc(bytes ? bytes : 1); }
void eprem_gpu_host_free(void *p) { free(p); }

int eprem_gpu_host_register(void *p, size_t bytes) {
  (void)p; (void)bytes;
  return EPREM_GPU_OK;
}
int eprem_gpu_host_unregister(void *p) {
  (void)p;
  return EPREM_GPU_OK;
}

int eprem_gpu_update_energetic_particles_host(eprem_gpu_run *r, const double *f_in,
                                              double *f_out, size_t stream_pitch,
                                              double t_global) {
  const size_t per = (size_t)r->d.num_nodes * r->d.num_energies * r->d.num_mu;
  const size_t pitch = stream_pitch ? stream_pitch : per;
  if (pitch < per) return abi_fail(EPREM_GPU_ERR_ARG, "stream_pitch below N*E*M");
  for (int s = 0; s < r->d.num_streams; s++)
    memcpy(r->f + (size_t)s * per, f_in + (size_t)s * pitch, per * sizeof(double));
  int rc = eprem_gpu_update_energetic_particles(r, t_global);
  if (rc == EPREM_GPU_OK)
    for (int s = 0; s < r->d.num_streams; s++)
      memcpy(f_out + (size_t)s * pitch, r->f + (size_t)s * per, per * sizeof(double));
  return rc;
}

int eprem_gpu_set_shell_diffusion(eprem_gpu_run *r, const int32_t *news, double kperxkpar) {
  free(r->news);
  r->news = NULL;
  if (!news) return EPREM_GPU_OK;
  if (!(kperxkpar >= 1.0e-33)) return abi_fail(EPREM_GPU_ERR_ARG, "kperxkpar below 1e-33");
  const size_t n = 4 * (size_t)r->d.num_streams;
  r->news = (int32_t *)malloc(n * sizeof(int32_t));
  memcpy(r->news, news, n * sizeof(int32_t));
  r->kperxkpar = kperxkpar;
  return EPREM_GPU_OK;
}

int eprem_gpu_read_stats(eprem_gpu_run *r, eprem_ep_stats_t *s) {
  *s = r->stats;
  stats_reset(&r->stats);
  return EPREM_GPU_OK;
}

int eprem_gpu_update_mhd(eprem_gpu_run *r, double t_global) {
  rec_call(r, REC_MHD, t_global);
  if (r->mas_on && r->drift_on)
    return abi_fail(EPREM_GPU_ERR_UNSUPPORTED, "drift with the MAS background");
  const int rc = r->mas_on ? orc_mas_update_mhd(&r->d, &r->p, r->nodes, &r->mas, t_global)
                 : r->drift_on ? orc_update_mhd_curl(&r->d, &r->p, r->nodes, t_global, r->curl)
                               : orc_update_mhd(&r->d, &r->p, r->nodes, t_global);
  return rc == EPREM_GPU_OK ? rc : abi_fail(rc, "updateMhd");
}

int eprem_gpu_set_drift(eprem_gpu_run *r, const int32_t *news, const eprem_drift_params_t *dp) {
  if (!dp) {
    r->drift_on = 0;
    return EPREM_GPU_OK;
  }
  if (r->mas_on) return abi_fail(EPREM_GPU_ERR_UNSUPPORTED, "drift with the MAS background");
  const size_t sn = (size_t)r->d.num_streams * r->d.num_nodes;
  if (!r->curl) r->curl = (double *)calloc(3 * sn, sizeof(double));
  r->drift = *dp;
  r->drift_on = 1;
  if (news) {
    const size_t n = 4 * (size_t)r->d.num_streams;
    free(r->drift_news);
    r->drift_news = (int32_t *)malloc(n * sizeof(int32_t));
    memcpy(r->drift_news, news, n * sizeof(int32_t));
  }
  return EPREM_GPU_OK;
}
int eprem_gpu_move_nodes(eprem_gpu_run *r, double dt) {
  rec_call(r, REC_MOVE, dt);
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
  rec_call(r, REC_MAS_MOVE, dt);
  const int rc = orc_mas_move_nodes(&r->d, &r->p, r->nodes, &r->mas, dt);
  return rc == EPREM_GPU_OK ? rc : abi_fail(rc, "masMoveNodes");
}
