/*
 * eprem_oracle.c -- CPU restatement of EPREM's per-timestep particle update.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker that tests/, smoke()
 * and bench.py's cpu_baseline leg compare the CUDA path against; the product
 * library never links or calls it.
 *
 * Every function restates one reference function (cited file:line, paths in
 * the predsci/eprem tree) keeping its operation order, so that with
 * -ffp-contract=off it reproduces the reference C bit for bit; the pinning
 * test runs both on the same states.  Layout: include/eprem_gpu.h.
 *
 * Restrictions (shared with the CUDA path): one species, one MPI rank's view
 * of whole streams, no MAS heliospheric switches, no drift / shell diffusion.
 */
#include "eprem_oracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* Physical constants, src/baseTypes.h:47-86. */
#define ORC_PI 3.1415926535897932
#define ORC_MP 1.6726e-24
#define ORC_MEV 1.6022e-6
#define ORC_GEV 1.6022e-3
#define ORC_C 2.99792458e10
#define ORC_AU 1.495978707e13
#define ORC_VERYSMALL 1.0e-33
#define ORC_MZERO (ORC_MP * ORC_C * ORC_C / ORC_GEV)
#define ORC_TAU (ORC_AU / ORC_C)
#define ORC_DAY (ORC_TAU / (24.0 * 60.0 * 60.0))
#define ORC_MHD_DENSITY_NORM 1.0
#define ORC_MHD_B_NORM (sqrt(ORC_MP * ORC_MHD_DENSITY_NORM) * ORC_C)
#define ORC_MAS_TIME_NORM 1445.87003080685

/* ------------------------------------------------------------------------ */
void orc_build_grids(int E, int M, double e_min_mev, double e_max_mev,
                     double mass, double charge, double rigidity_power,
                     double *egrid, double *vgrid, double *vgrid_i,
                     double *pgrid, double *rigidity, double *mugrid,
                     double *dlnp_out, double *dmu_out) {
  /* src/energeticParticlesInit.c:52-89 */
  const double one = 1.0, two = 2.0, half = 0.5;
  double kin = e_min_mev * ORC_MEV / (ORC_MP * ORC_C * ORC_C);
  double lnpmin = log(sqrt(kin * kin + two * kin));
  kin = e_max_mev * ORC_MEV / (ORC_MP * ORC_C * ORC_C);
  double lnpmax = log(sqrt(kin * kin + two * kin));
  double dlnp = (lnpmax - lnpmin) / (E - 1.0);
  for (int e = 0; e < E; e++) {
    double p = exp(lnpmin + e * dlnp);
    pgrid[e] = p;
    egrid[e] = sqrt(one + p * p) - one;
    vgrid[e] = p / sqrt(one + p * p);
    vgrid_i[e] = sqrt(one + p * p) / p;
  }
  for (int e = 0; e < E; e++) {
    double p = exp(lnpmin + e * dlnp);
    rigidity[e] = (mass / charge) * p * ORC_MZERO;
    rigidity[e] = pow(rigidity[e], rigidity_power);
  }
  double dmu = two / (one * M);
  for (int m = 0; m < M; m++) {
    double mup = -one + (m + one) * dmu;
    double mum = -one + m * dmu;
    mugrid[m] = half * (mup + mum);
  }
  *dlnp_out = dlnp;
  *dmu_out = dmu;
}

void orc_default_params(eprem_params_t *p) {
  /* getParams defaults (src/configuration.c:58-217) converted as in
   * setRuntimeConstants (:325-348). */
  memset(p, 0, sizeof(*p));
  p->r_scale = 0.005;
  p->t_del = 0.01041666666667 / ORC_DAY;
  p->num_ep_steps = 30;
  p->use_parallel_diffusion = 1;
  p->use_adiabatic_focus = 1;
  p->use_adiabatic_change = 1;
  p->check_seed_population = 1;
  p->use_ep_boundary = 1;
  p->use_boundary_function = 1;
  p->adiabatic_focus_alg = 1;
  p->adiabatic_change_alg = 1;
  p->damp_cooling = 0.0;
  p->dsh_min = 5.0e-5;
  p->mfp_type = 1;
  p->lamo = 1.0;
  p->mfp_radial_power = 2.0;
  p->mfp_b_power = 0.75;
  p->mhd_bs_au = 1.60e-5 / ORC_MHD_B_NORM;
  p->bf_amplitude = 1.0;
  p->bf_xi = 1.0;
  p->bf_gamma = 2.0;
  p->bf_beta = 1.7;
  p->bf_ecutoff = 1.0;
  p->bf_r0 = 1.0;
  p->mhd_us = 400.0e5 / ORC_C;
  p->mhd_ns_au = 8.30 / ORC_MHD_DENSITY_NORM;
  p->omega_sun = (0.004144 / ORC_MAS_TIME_NORM) * ORC_TAU;
  p->ideal_shock = 0;
  p->ideal_shock_sharpness = 1.0;
  p->ideal_shock_scale_length = 0.0046491;
  p->ideal_shock_jump = 4.0;
  p->ideal_shock_falloff = 0.0;
  p->ideal_shock_speed = 1500e5;
  p->ideal_shock_init_time = 0.0;
  p->ideal_shock_theta = 1.570796;
  p->ideal_shock_phi = 0.0;
  p->ideal_shock_width = 0.0;
  p->max_subcycles = 0;
}

/* sepSeedFunction, src/energeticParticlesBoundary.c:67-116. */
double orc_seed_function(const eprem_params_t *p, double energy, double r) {
  const double two = 2.0;
  const double E1 = 1.0;
  const double efac = ORC_MEV / (ORC_MP * ORC_C * ORC_C);
  double normJ0 = p->bf_amplitude * (ORC_MP * ORC_C) / (ORC_MHD_DENSITY_NORM * ORC_MEV);
  double normRadius = p->bf_r0 / p->r_scale;
  double normE1 = E1 * efac;
  double normE0 = p->bf_ecutoff * efac;
  double radialTerm = pow((r / normRadius), -p->bf_beta);
  double powerLawTerm = pow((energy / normE1), -p->bf_gamma);
  double expTerm = exp(-(energy / normE0));
  double normJHe = normJ0 * radialTerm * powerLawTerm * expTerm;
  double normJ = normJHe / p->bf_xi;
  double normf = normJ / (two * energy);
  if (normf < DBL_MIN) normf = DBL_MIN;
  return normf;
}

/* meanFreePath, src/meanFreePath.c:13-50 (mfpType 1 or 2). */
static double orc_mfp(const eprem_params_t *p, const eprem_grids_t *g, int e,
                      double rmag, double bmag) {
  if (p->mfp_type == 2)
    return g->rigidity[e] * p->lamo * pow(p->mhd_bs_au / bmag, p->mfp_b_power);
  return g->rigidity[e] * p->lamo * pow(rmag * p->r_scale, p->mfp_radial_power);
}

/* ------------------------------------------------------------------------ */
/* Per-stream working storage (the reference's streamGrid/shellList/... globals
 * of src/global.c:21-33, one set per worker thread). */
typedef struct {
  int *list, *ref;
  double *ds_list, *ds_i;
  double *f_old, *f_new, *iso, *mult, *emt, *del_fac;
  double *nf, *nf1, *nvel, *nvavg, *ns1, *nflux, *nLP, *nLN, *nalpha;
} orc_work_t;

typedef struct {
  const eprem_dims_t *d;
  const eprem_params_t *p;
  const eprem_grids_t *g;
  double *f, *nodes;
  int s0, s1;
  int step0, step1;  /* sub-steps [step0, step1) of the call */
  eprem_ep_stats_t stats;
  int status;
  char err[256];
} orc_job_t;

#define NODE(field, s, k) nodes[(size_t)(field) * SN + (size_t)(s) * N + (k)]
#define FIDX(s, k, e, m) ((((size_t)(s) * N + (k)) * E + (e)) * M + (m))

static int orc_fail(orc_job_t *job, int code, const char *what, int s, int k) {
  if (job->status == EPREM_GPU_OK) {
    job->status = code;
    snprintf(job->err, sizeof(job->err), "%s in %s (stream %d, node %d)",
             code == EPREM_GPU_ERR_NAN   ? "NaN value"
             : code == EPREM_GPU_ERR_INF ? "Inf value"
                                         : "failure",
             what, s, k);
  }
  return code;
}

static int orc_check(orc_job_t *job, double v, const char *what, int s, int k) {
  /* checkNaN / checkInf, src/error.c:57-102 */
  if (isnan(v)) return orc_fail(job, EPREM_GPU_ERR_NAN, what, s, k);
  if (isinf(v)) return orc_fail(job, EPREM_GPU_ERR_INF, what, s, k);
  return EPREM_GPU_OK;
}

/* updateStreamValues, src/simCore.c:326-435. */
static void orc_stream_values(orc_job_t *job, int s) {
  const int N = job->d->num_nodes;
  const size_t SN = (size_t)job->d->num_streams * N;
  double *nodes = job->nodes;
  const double rs = job->p->r_scale;
  for (int k = 0; k < N; k++) {
    double rx = NODE(EPREM_NODE_RX, s, k) * rs, ry = NODE(EPREM_NODE_RY, s, k) * rs,
           rz = NODE(EPREM_NODE_RZ, s, k) * rs;
    if (k == 0) {
      double px = NODE(EPREM_NODE_RX, s, k + 1) * rs, py = NODE(EPREM_NODE_RY, s, k + 1) * rs,
             pz = NODE(EPREM_NODE_RZ, s, k + 1) * rs;
      NODE(EPREM_NODE_DS, s, k) =
          sqrt((px - rx) * (px - rx) + (py - ry) * (py - ry) + (pz - rz) * (pz - rz));
      NODE(EPREM_NODE_BMAG_MINUS, s, k) = NODE(EPREM_NODE_BMAG, s, k);
      NODE(EPREM_NODE_BMAG_PLUS, s, k) = NODE(EPREM_NODE_BMAG, s, k + 1);
    } else if (k == N - 1) {
      double mx = NODE(EPREM_NODE_RX, s, k - 1) * rs, my = NODE(EPREM_NODE_RY, s, k - 1) * rs,
             mz = NODE(EPREM_NODE_RZ, s, k - 1) * rs;
      NODE(EPREM_NODE_DS, s, k) =
          sqrt((rx - mx) * (rx - mx) + (ry - my) * (ry - my) + (rz - mz) * (rz - mz));
      NODE(EPREM_NODE_BMAG_MINUS, s, k) = NODE(EPREM_NODE_BMAG, s, k - 1);
      NODE(EPREM_NODE_BMAG_PLUS, s, k) = NODE(EPREM_NODE_BMAG, s, k);
    } else {
      double px = NODE(EPREM_NODE_RX, s, k + 1) * rs, py = NODE(EPREM_NODE_RY, s, k + 1) * rs,
             pz = NODE(EPREM_NODE_RZ, s, k + 1) * rs;
      double mx = NODE(EPREM_NODE_RX, s, k - 1) * rs, my = NODE(EPREM_NODE_RY, s, k - 1) * rs,
             mz = NODE(EPREM_NODE_RZ, s, k - 1) * rs;
      double dsPlus = sqrt((px - rx) * (px - rx) + (py - ry) * (py - ry) + (pz - rz) * (pz - rz));
      double dsMinus = sqrt((rx - mx) * (rx - mx) + (ry - my) * (ry - my) + (rz - mz) * (rz - mz));
      NODE(EPREM_NODE_DS, s, k) = 0.5 * (dsPlus + dsMinus);
      NODE(EPREM_NODE_BMAG_MINUS, s, k) = NODE(EPREM_NODE_BMAG, s, k - 1);
      NODE(EPREM_NODE_BMAG_PLUS, s, k) = NODE(EPREM_NODE_BMAG, s, k + 1);
    }
  }
}

/* seedPopulationCheck, src/energeticParticlesBoundary.c:28-59. */
static void orc_seed_check(orc_job_t *job, int s) {
  const int N = job->d->num_nodes, E = job->d->num_energies, M = job->d->num_mu;
  const size_t SN = (size_t)job->d->num_streams * N;
  double *nodes = job->nodes, *f = job->f;
  for (int k = 0; k < N; k++)
    for (int e = 0; e < E; e++) {
      double seed = orc_seed_function(job->p, job->g->egrid[e], NODE(EPREM_NODE_RMAG, s, k));
      for (int m = 0; m < M; m++)
        if (f[FIDX(s, k, e, m)] < seed) f[FIDX(s, k, e, m)] = seed;
    }
}

static double orc_dist(const double *nodes, size_t SN, int N, int s, int a, int b,
                       double rs) {
  /* |r_a - r_b| with positions scaled to AU first, summed x,y,z in order as in
   * src/energeticParticles.c:2193-2203 and :2519-2529. */
  double ax = NODE(EPREM_NODE_RX, s, a) * rs, ay = NODE(EPREM_NODE_RY, s, a) * rs,
         az = NODE(EPREM_NODE_RZ, s, a) * rs;
  double bx = NODE(EPREM_NODE_RX, s, b) * rs, by = NODE(EPREM_NODE_RY, s, b) * rs,
         bz = NODE(EPREM_NODE_RZ, s, b) * rs;
  return sqrt((ax - bx) * (ax - bx) + (ay - by) * (ay - by) + (az - bz) * (az - bz));
}

/* GetStreamList (src/energeticParticles.c:2150-2234) and FindSegmentLengths
 * (:2496-2601).  Returns the list size, or a negative status. */
static int orc_stream_list(orc_job_t *job, orc_work_t *w, int s, double *dsMin_out) {
  const int N = job->d->num_nodes;
  const size_t SN = (size_t)job->d->num_streams * N;
  const double *nodes = job->nodes;
  const double rs = job->p->r_scale;
  const double dshmin = job->p->dsh_min;
  int L = 0, down = 0, up;
  for (int shell = 0; shell < N; shell++) {
    if (shell < N - 1) {
      up = shell + 1;
    } else {
      up = shell;
      down = shell - 1;
    }
    double dsh = orc_dist(nodes, SN, N, s, up, down, rs);
    if ((dsh > dshmin) || (shell == N - 1)) {
      w->list[L++] = shell;
      w->ref[shell] = shell;
      down = shell + 1;
    } else {
      w->ref[shell] = shell + 1;
      int sp = shell - 1;
      while ((sp >= 0) && (w->ref[sp] != sp)) {
        w->ref[sp] = w->ref[sp + 1];
        sp--;
      }
    }
  }
  if (L < 3) {
    orc_fail(job, EPREM_GPU_ERR_STATE, "GetStreamList (fewer than 3 nodes kept)", s, L);
    return EPREM_GPU_ERR_STATE;
  }
  double dsMin = 10000.0 * rs;
  for (int sl = 0; sl < L; sl++) {
    int th = w->list[sl];
    if (sl == 0) {
      double dsh = orc_dist(nodes, SN, N, s, w->list[sl + 1], th, rs);
      if (dsh < dsMin) dsMin = dsh;
      w->ds_list[sl] = dsh;
    } else if (sl == L - 1) {
      double dsh = orc_dist(nodes, SN, N, s, th, w->list[sl - 1], rs);
      if (dsh < dsMin) dsMin = dsh;
      w->ds_list[sl] = dsh;
    } else {
      double ds1 = orc_dist(nodes, SN, N, s, w->list[sl + 1], th, rs);
      double ds9 = orc_dist(nodes, SN, N, s, th, w->list[sl - 1], rs);
      if (ds1 < dsMin) dsMin = ds1;
      if (ds9 < dsMin) dsMin = ds9;
      w->ds_list[sl] = 0.5 * (ds1 + ds9);
    }
    if (dsMin <= 0.0) {
      orc_fail(job, EPREM_GPU_ERR_DS, "FindSegmentLengths(): Underflow in ds", s, th);
      return EPREM_GPU_ERR_DS;
    }
    w->ds_i[sl] = 1.0 / w->ds_list[sl];
  }
  *dsMin_out = dsMin;
  return L;
}

/* DiffuseStreamData, src/energeticParticles.c:2240-2490 (species 0). */
static int orc_diffuse_stream(orc_job_t *job, orc_work_t *w, int s, int L, double dsMin,
                              double dt) {
  const eprem_params_t *p = job->p;
  const eprem_grids_t *g = job->g;
  const int N = job->d->num_nodes, E = job->d->num_energies, M = job->d->num_mu;
  const size_t SN = (size_t)job->d->num_streams * N;
  double *nodes = job->nodes, *f = job->f;
  const double one = 1.0;
  const double NUM_MUSTEPS_I = one / M;
  const int cap = p->max_subcycles > 0 ? p->max_subcycles : 1000000;
  double *f_old = w->f_old, *f_new = w->f_new, *iso_vec = w->iso;
  double sep_seed_vec[3];
  for (int e = 0; e < E; e++) {
    double v = g->vgrid[e], vi = g->vgrid_i[e];
    double dtMin = 0.4 * dsMin * vi;
    double nst = floor(dt / dtMin + one);
    if (!(nst <= (double)cap))
      return orc_fail(job, EPREM_GPU_ERR_SUBCYCLES, "DiffuseStreamData", s, e);
    int nsteps = (int)nst;
    if (nsteps > job->stats.max_substeps_stream) job->stats.max_substeps_stream = nsteps;
    double dtProp = dt / (one * nsteps);
    double dtProp_i = one / dtProp;
    for (int sl = 0; sl < L; sl++) {
      int sh = w->list[sl];
      double tau = vi * orc_mfp(p, g, e, NODE(EPREM_NODE_RMAG, s, sh), NODE(EPREM_NODE_BMAG, s, sh));
      if (dtProp > tau)
        w->mult[sl] = w->ds_i[sl] * tau * dtProp_i;
      else
        w->mult[sl] = w->ds_i[sl] * one;
      w->emt[sl] = exp(-dtProp / tau);
    }
    for (int sl = 0; sl < 3; sl++)
      sep_seed_vec[sl] = orc_seed_function(p, g->egrid[e], NODE(EPREM_NODE_RMAG, s, w->list[sl]));
    for (int m = 0; m < M; m++) w->del_fac[m] = v * dtProp * g->mugrid[m];
    for (int m = 0; m < M; m++)
      for (int sl = 0; sl < L; sl++) f_old[(size_t)L * m + sl] = f[FIDX(s, w->list[sl], e, m)];
    for (int step = 0; step < nsteps; step++) {
      if ((p->use_ep_boundary > 0) && (p->use_boundary_function > 0))
        for (int m = 0; m < M; m++)
          for (int sl = 0; sl < 3; sl++) f_old[(size_t)L * m + sl] = sep_seed_vec[sl];
      for (int m = 0; m < M; m++) {
        double del_fac = w->del_fac[m];
        double *fo = f_old + (size_t)L * m, *fn = f_new + (size_t)L * m;
        if (g->mugrid[m] >= 0.0) {
          fn[0] = fo[0];
          for (int sl = 1; sl < L; sl++)
            fn[sl] = fo[sl] + w->mult[sl] * del_fac * (fo[sl - 1] - fo[sl]);
        } else {
          fn[L - 1] = fo[L - 1];
          for (int sl = 0; sl < L - 1; sl++)
            fn[sl] = fo[sl] + w->mult[sl] * del_fac * (fo[sl] - fo[sl + 1]);
        }
      }
      for (int sl = 0; sl < L; sl++) iso_vec[sl] = 0.0;
      for (int m = 0; m < M; m++)
        for (int sl = 0; sl < L; sl++) iso_vec[sl] = iso_vec[sl] + f_new[(size_t)L * m + sl];
      for (int m = 0; m < M; m++)
        for (int sl = 0; sl < L; sl++) {
          double iso = NUM_MUSTEPS_I * iso_vec[sl];
          f_old[(size_t)L * m + sl] = iso + (f_new[(size_t)L * m + sl] - iso) * w->emt[sl];
        }
    }
    job->stats.stream_cell_subcycles += (double)nsteps * L * M;
    for (int m = 0; m < M; m++)
      for (int sl = 0; sl < L; sl++) f[FIDX(s, w->list[sl], e, m)] = f_old[(size_t)L * m + sl];
    for (int m = 0; m < M; m++)
      for (int sh = 0; sh < N; sh++) {
        if (sh != w->ref[sh]) f[FIDX(s, sh, e, m)] = f[FIDX(s, w->ref[sh], e, m)];
        double val = f[FIDX(s, sh, e, m)];
        if (orc_check(job, val, "Diffuse Stream Data", s, sh)) return job->status;
        if (val < DBL_MIN) f[FIDX(s, sh, e, m)] = DBL_MIN;
      }
  }
  return EPREM_GPU_OK;
}

/* AdiabaticFocusing_Operator_Upwind, src/energeticParticles.c:1809-1895, for
 * one node: f, f1 [E][M]; v_avg [E][M+1]. */
static void orc_focus_op_upwind(double *f1, const double *f, const double *v_avg,
                                double *flux, int E, int M, double dmu) {
  const double upwind = 1.0;
  double dmu_i = 1.0 / dmu;
  for (int e = 0; e < E; e++)
    for (int m = 1; m < M; m++) {
      double va = v_avg[e * (M + 1) + m];
      double cce = copysign(upwind, va);
      flux[e * (M + 1) + m] = va * 0.5 * ((1.0 - cce) * f[e * M + m] + (1.0 + cce) * f[e * M + m - 1]);
    }
  for (int e = 0; e < E; e++)
    for (int m = 1; m < M - 1; m++)
      f1[e * M + m] = (flux[e * (M + 1) + m + 1] - flux[e * (M + 1) + m]) * dmu_i;
  for (int e = 0; e < E; e++) {
    double va = v_avg[e * (M + 1) + 1];
    if (va <= 0)
      f1[e * M + 0] = va * f[e * M + 1] * dmu_i;
    else
      f1[e * M + 0] = va * f[e * M + 0] * dmu_i;
    va = v_avg[e * (M + 1) + M - 1];
    if (va >= 0)
      f1[e * M + M - 1] = va * (-f[e * M + M - 2]) * dmu_i;
    else
      f1[e * M + M - 1] = va * (-f[e * M + M - 1]) * dmu_i;
  }
}

/* WENO3 building blocks shared by both operators
 * (src/energeticParticles.c:1311-1346 and :2031-2066). */
static double orc_weno_flux(double LNm2, double LNm1, double LN0, double LP_1, double LP0,
                            double LPp1, double cc, double cp, double mt, double cpt,
                            double pt, double mct, double eps) {
  /* cc = D_C_CPt, (...) names follow the reference's D_* constants */
  double D_C_CPt = cc, D_C_MCt = cp, D_M_Tt = mt, D_CP_Tt = cpt, D_P_Tt = pt, D_MC_Tt = mct;
  double p0m = (1.0 + D_C_MCt) * LNm1 - D_C_MCt * LNm2;
  double p1m = D_C_MCt * LNm1 + D_C_CPt * LN0;
  double p0p = (1.0 + D_C_CPt) * LP0 - D_C_CPt * LPp1;
  double p1p = D_C_CPt * LP0 + D_C_MCt * LP_1;
  double B0m = 4.0 * pow((D_C_MCt * (LNm1 - LNm2)), 2);
  double B1m = 4.0 * pow((D_C_CPt * (LN0 - LNm1)), 2);
  double B0p = 4.0 * pow((D_C_CPt * (LPp1 - LP0)), 2);
  double B1p = 4.0 * pow((D_C_MCt * (LP0 - LP_1)), 2);
  double w0m = D_P_Tt / pow((eps + B0m), 2);
  double w1m = D_MC_Tt / pow((eps + B1m), 2);
  double w0p = D_M_Tt / pow((eps + B0p), 2);
  double w1p = D_CP_Tt / pow((eps + B1p), 2);
  double wm_sum = w0m + w1m;
  double wp_sum = w0p + w1p;
  double OM0m = w0m / wm_sum, OM1m = w1m / wm_sum, OM0p = w0p / wp_sum, OM1p = w1p / wp_sum;
  double um = OM0m * p0m + OM1m * p1m;
  double up = OM0p * p0p + OM1p * p1p;
  return up + um;
}

/* max |v| over v_avg[i] for i in [lo, hi] (inclusive), the alpha of the WENO3
 * operators; max is order-independent so the reference's unrolled
 * comparisons (:1237-1295, :1957-2015) reduce to this. */
static double orc_alpha(const double *va, int stride, int lo, int hi) {
  double a = 0.0;
  for (int i = lo; i <= hi; i++) {
    double x = fabs(va[i * stride]);
    if (i == lo || x > a) a = x;
  }
  return a;
}

/* AdiabaticFocusing_Operator_WENO3, src/energeticParticles.c:1902-2144. */
static void orc_focus_op_weno3(double *f1, const double *f, const double *v_avg, double *flux,
                               double *LP, double *LN, double *alpha, int E, int M, double dmu) {
  const double upwind = 1.0;
  const double D_C_CPt = 1 / 2.0, D_C_MCt = 1 / 2.0, D_M_Tt = 1 / 3.0, D_CP_Tt = 2 / 3.0,
               D_P_Tt = 1 / 3.0, D_MC_Tt = 2 / 3.0;
  const double weno_eps = 10.0 * sqrt(DBL_MIN);
  for (int e = 0; e < E; e++) {
    const double *va = v_avg + e * (M + 1);
    for (int m = 2; m < M - 2; m++) alpha[e * M + m] = orc_alpha(va, 1, m - 2, m + 3);
    alpha[e * M + 0] = orc_alpha(va, 1, 0, 3);
    alpha[e * M + 1] = orc_alpha(va, 1, 0, 4);
    alpha[e * M + M - 2] = orc_alpha(va, 1, M - 4, M);
    alpha[e * M + M - 1] = orc_alpha(va, 1, M - 3, M);
  }
  for (int e = 0; e < E; e++)
    for (int m = 0; m < M; m++) {
      LP[e * M + m] = 0.5 * f[e * M + m] * v_avg[e * (M + 1) + m + 1] - alpha[e * M + m];
      LN[e * M + m] = 0.5 * f[e * M + m] * v_avg[e * (M + 1) + m] + alpha[e * M + m];
    }
  for (int e = 0; e < E; e++)
    for (int m = 2; m < M - 1; m++) {
      const double *ln = LN + e * M, *lp = LP + e * M;
      flux[e * (M + 1) + m] = orc_weno_flux(ln[m - 2], ln[m - 1], ln[m], lp[m - 1], lp[m], lp[m + 1],
                                            D_C_CPt, D_C_MCt, D_M_Tt, D_CP_Tt, D_P_Tt, D_MC_Tt,
                                            weno_eps);
    }
  for (int e = 0; e < E; e++) {
    int m = 1;
    double va = v_avg[e * (M + 1) + m];
    double cce = copysign(upwind, va);
    flux[e * (M + 1) + m] = va * 0.5 * ((1.0 - cce) * f[e * M + m] + (1.0 + cce) * f[e * M + m - 1]);
    m = M - 1;
    va = v_avg[e * (M + 1) + m];
    cce = copysign(upwind, va);
    flux[e * (M + 1) + m] = va * 0.5 * ((1.0 - cce) * f[e * M + m] + (1.0 + cce) * f[e * M + m - 1]);
  }
  for (int e = 0; e < E; e++)
    for (int m = 1; m < M - 1; m++)
      f1[e * M + m] = (flux[e * (M + 1) + m + 1] - flux[e * (M + 1) + m]) / dmu;
  for (int e = 0; e < E; e++) {
    double va = v_avg[e * (M + 1) + 1];
    if (va <= 0)
      f1[e * M + 0] = va * f[e * M + 1] / dmu;
    else
      f1[e * M + 0] = va * f[e * M + 0] / dmu;
    va = v_avg[e * (M + 1) + M - 1];
    if (va >= 0)
      f1[e * M + M - 1] = va * (-f[e * M + M - 2]) / dmu;
    else
      f1[e * M + M - 1] = va * (-f[e * M + M - 1]) / dmu;
  }
}

/* One RK3-TVD or Euler advance of f over n sub-cycles of length dts, with the
 * operator chosen by alg, as in the sub-cycle loops of AdiabaticFocusing
 * (:1677-1763) and AdiabaticChange (:952-1038). */
typedef void (*orc_op_fn)(void *ctx, double *f1, const double *f);

static void orc_subcycle(int alg, int n, double dts, double *f, double *f1, double *s1,
                         int cells, orc_op_fn op, void *ctx) {
  if (alg == 2 || alg == 3) {
    for (int s = 0; s < n; s++) {
      op(ctx, f1, f);
      for (int i = 0; i < cells; i++) s1[i] = f[i] - dts * f1[i];
      op(ctx, f1, s1);
      for (int i = 0; i < cells; i++)
        s1[i] = (3.0 / 4.0) * f[i] + (1.0 / 4.0) * s1[i] - (1.0 / 4.0) * dts * f1[i];
      op(ctx, f1, s1);
      for (int i = 0; i < cells; i++)
        f[i] = (1.0 / 3.0) * f[i] + (2.0 / 3.0) * s1[i] - (2.0 / 3.0) * dts * f1[i];
    }
  } else {
    for (int s = 0; s < n; s++) {
      op(ctx, f1, f);
      for (int i = 0; i < cells; i++) f[i] = f[i] - dts * f1[i];
    }
  }
}

typedef struct {
  orc_work_t *w;
  int alg, E, M;
  double d;           /* dmu or dlnp */
  double bc0, bc1;    /* change only: log seed at E0 and E_last */
  const eprem_params_t *p;
  const eprem_grids_t *g;
  double rmag;
} orc_opctx_t;

static void orc_focus_op(void *vctx, double *f1, const double *f) {
  orc_opctx_t *c = (orc_opctx_t *)vctx;
  if (c->alg == 3)
    orc_focus_op_weno3(f1, f, c->w->nvavg, c->w->nflux, c->w->nLP, c->w->nLN, c->w->nalpha,
                       c->E, c->M, c->d);
  else
    orc_focus_op_upwind(f1, f, c->w->nvavg, c->w->nflux, c->E, c->M, c->d);
}

/* AdiabaticChange_Operator_Upwind, src/energeticParticles.c:1084-1176:
 * arrays [E][M], v_avg [E+1][M]. */
static void orc_change_op_upwind(double *f1, const double *f, const double *v_avg, double *flux,
                                 int E, int M, double dlnp, double bc_val0, double bc_val1) {
  const double upwind = 1.0;
  double dlnp_i = 1.0 / dlnp;
  for (int e = 1; e < E; e++)
    for (int m = 0; m < M; m++) {
      double va = v_avg[e * M + m];
      double cce = copysign(upwind, va);
      flux[e * M + m] = va * 0.5 * ((1.0 - cce) * f[e * M + m] + (1.0 + cce) * f[(e - 1) * M + m]);
    }
  for (int e = 1; e < E - 1; e++)
    for (int m = 0; m < M; m++)
      f1[e * M + m] = (flux[(e + 1) * M + m] - flux[e * M + m]) * dlnp_i;
  for (int m = 0; m < M; m++) {
    double va = v_avg[1 * M + m];
    if (va <= 0)
      f1[m] = va * (f[1 * M + m] - f[m]) * dlnp_i;
    else
      f1[m] = va * (f[m] - bc_val0) * dlnp_i;
    va = v_avg[(E - 1) * M + m];
    if (va >= 0)
      f1[(E - 1) * M + m] = va * (f[(E - 1) * M + m] - f[(E - 2) * M + m]) * dlnp_i;
    else
      f1[(E - 1) * M + m] = va * (bc_val1 - f[(E - 1) * M + m]) * dlnp_i;
  }
}

/* AdiabaticChange_Operator_WENO3, src/energeticParticles.c:1182-1427. */
static void orc_change_op_weno3(double *f1, const double *f, const double *v_avg, double *flux,
                                double *LP, double *LN, double *alpha, int E, int M, double dlnp,
                                double bc_val0, double bc_val1) {
  const double upwind = 1.0;
  const double D_C_CPt = 0.5, D_C_MCt = 0.5, D_M_Tt = 1.0 / 3.0, D_CP_Tt = 2.0 / 3.0,
               D_P_Tt = 1.0 / 3.0, D_MC_Tt = 2.0 / 3.0;
  const double weno_eps = 10.0 * sqrt(DBL_MIN);
  for (int m = 0; m < M; m++) {
    const double *va = v_avg + m;
    for (int e = 2; e < E - 2; e++) alpha[e * M + m] = orc_alpha(va, M, e - 2, e + 3);
    alpha[0 * M + m] = orc_alpha(va, M, 0, 3);
    alpha[1 * M + m] = orc_alpha(va, M, 0, 4);
    alpha[(E - 2) * M + m] = orc_alpha(va, M, E - 4, E);
    alpha[(E - 1) * M + m] = orc_alpha(va, M, E - 3, E);
  }
  for (int e = 0; e < E; e++)
    for (int m = 0; m < M; m++) {
      LP[e * M + m] = 0.5 * f[e * M + m] * v_avg[(e + 1) * M + m] - alpha[e * M + m];
      LN[e * M + m] = 0.5 * f[e * M + m] * v_avg[e * M + m] + alpha[e * M + m];
    }
  for (int e = 2; e < E - 1; e++)
    for (int m = 0; m < M; m++)
      flux[e * M + m] = orc_weno_flux(LN[(e - 2) * M + m], LN[(e - 1) * M + m], LN[e * M + m],
                                      LP[(e - 1) * M + m], LP[e * M + m], LP[(e + 1) * M + m],
                                      D_C_CPt, D_C_MCt, D_M_Tt, D_CP_Tt, D_P_Tt, D_MC_Tt, weno_eps);
  for (int m = 0; m < M; m++) {
    int e = 1;
    double va = v_avg[e * M + m];
    double cce = copysign(upwind, va);
    flux[e * M + m] = va * 0.5 * ((1.0 - cce) * f[e * M + m] + (1.0 + cce) * f[(e - 1) * M + m]);
    e = E - 1;
    va = v_avg[e * M + m];
    cce = copysign(upwind, va);
    flux[e * M + m] = va * 0.5 * ((1.0 - cce) * f[e * M + m] + (1.0 + cce) * f[(e - 1) * M + m]);
  }
  for (int e = 1; e < E - 1; e++)
    for (int m = 0; m < M; m++) f1[e * M + m] = (flux[(e + 1) * M + m] - flux[e * M + m]) / dlnp;
  for (int m = 0; m < M; m++) {
    double va = v_avg[1 * M + m];
    if (va <= 0)
      f1[m] = va * (f[1 * M + m] - f[m]) / dlnp;
    else
      f1[m] = va * (f[m] - bc_val0) / dlnp;
    va = v_avg[(E - 1) * M + m];
    if (va >= 0)
      f1[(E - 1) * M + m] = va * (f[(E - 1) * M + m] - f[(E - 2) * M + m]) / dlnp;
    else
      f1[(E - 1) * M + m] = va * (bc_val1 - f[(E - 1) * M + m]) / dlnp;
  }
}

static void orc_change_op(void *vctx, double *f1, const double *f) {
  orc_opctx_t *c = (orc_opctx_t *)vctx;
  if (c->alg == 3)
    orc_change_op_weno3(f1, f, c->w->nvavg, c->w->nflux, c->w->nLP, c->w->nLN, c->w->nalpha, c->E,
                        c->M, c->d, c->bc0, c->bc1);
  else
    orc_change_op_upwind(f1, f, c->w->nvavg, c->w->nflux, c->E, c->M, c->d, c->bc0, c->bc1);
}

/* AdiabaticFocusing for one node, src/energeticParticles.c:1581-1792. */
static int orc_focus_node(orc_job_t *job, orc_work_t *w, int s, int k, double dt) {
  const eprem_params_t *p = job->p;
  const eprem_grids_t *g = job->g;
  const int N = job->d->num_nodes, E = job->d->num_energies, M = job->d->num_mu;
  const size_t SN = (size_t)job->d->num_streams * N;
  double *nodes = job->nodes, *f = job->f;
  const double safety_factor = 0.9, half = 0.5, one = 1.0, two = 2.0, three = 3.0;
  const int cap = p->max_subcycles > 0 ? p->max_subcycles : 1000000;
  double dt_full = dt * p->num_ep_steps;
  double DuParDt = NODE(EPREM_NODE_DUPAR, s, k) / dt_full;
  double b = two * (NODE(EPREM_NODE_DLNN, s, k) / dt_full) - three * (NODE(EPREM_NODE_DLNB, s, k) / dt_full);
  double bp = NODE(EPREM_NODE_BMAG_PLUS, s, k), bm = NODE(EPREM_NODE_BMAG_MINUS, s, k);
  double dlnBds;
  if ((bp == 0.0) || (bm == 0.0))
    dlnBds = 0.0;
  else
    dlnBds = (log(bp) - log(bm)) / (two * NODE(EPREM_NODE_DS, s, k) + DBL_MIN);
  double vel_abs_max = 0.0;
  double *fn = w->nf, *vel = w->nvel, *v_avg = w->nvavg;
  for (int e = 0; e < E; e++)
    for (int m = 0; m < M; m++) {
      fn[e * M + m] = f[FIDX(s, k, e, m)];
      double muval = g->mugrid[m];
      double a = -g->vgrid[e] * dlnBds - (two / g->vgrid[e]) * DuParDt;
      vel[e * M + m] = half * (one - muval * muval) * (a + muval * b);
    }
  for (int e = 0; e < E; e++)
    for (int m = 0; m < M - 1; m++) {
      double va = half * (vel[e * M + m + 1] + vel[e * M + m]);
      v_avg[e * (M + 1) + m + 1] = va;
      if (fabs(va) > vel_abs_max) vel_abs_max = fabs(va);
    }
  for (int e = 0; e < E; e++) {
    v_avg[e * (M + 1) + 0] = v_avg[e * (M + 1) + 1];
    v_avg[e * (M + 1) + M] = v_avg[e * (M + 1) + M - 1];
  }
  double dt_stable = safety_factor * g->dmu / vel_abs_max;
  double nsub = ceil(dt / dt_stable);
  if (!(nsub <= (double)cap))
    return orc_fail(job, EPREM_GPU_ERR_SUBCYCLES, "Adiabatic Focusing", s, k);
  int N_sub = (int)nsub;
  if (N_sub > job->stats.max_subcycles_focusing) job->stats.max_subcycles_focusing = N_sub;
  double dt_sub = dt / N_sub;
  orc_opctx_t ctx = {w, p->adiabatic_focus_alg, E, M, g->dmu, 0.0, 0.0, p, g, 0.0};
  orc_subcycle(p->adiabatic_focus_alg, N_sub, dt_sub, fn, w->nf1, w->ns1, E * M, orc_focus_op, &ctx);
  job->stats.focus_cell_subcycles += (double)N_sub * E * M;
  for (int e = 0; e < E; e++)
    for (int m = 0; m < M; m++) {
      double val = fn[e * M + m];
      f[FIDX(s, k, e, m)] = val;
      if (orc_check(job, val, "Adiabatic Focusing", s, k)) return job->status;
      if (val < DBL_MIN) f[FIDX(s, k, e, m)] = DBL_MIN;
    }
  return EPREM_GPU_OK;
}

/* AdiabaticChange for one node, src/energeticParticles.c:843-1069. */
static int orc_change_node(orc_job_t *job, orc_work_t *w, int s, int k, double dt) {
  const eprem_params_t *p = job->p;
  const eprem_grids_t *g = job->g;
  const int N = job->d->num_nodes, E = job->d->num_energies, M = job->d->num_mu;
  const size_t SN = (size_t)job->d->num_streams * N;
  double *nodes = job->nodes, *f = job->f;
  const double safety_factor = 0.9, half = 0.5, one = 1.0;
  const int cap = p->max_subcycles > 0 ? p->max_subcycles : 1000000;
  double vel_abs_max = 0.0;
  double dt_full = dt * p->num_ep_steps;
  double DlnBDt = NODE(EPREM_NODE_DLNB, s, k) / dt_full;
  double DlnNDt = NODE(EPREM_NODE_DLNN, s, k) / dt_full;
  double cool_damp_fac = (DlnNDt < 0) ? 1.0 - p->damp_cooling : 1.0;
  double DuParDt = NODE(EPREM_NODE_DUPAR, s, k) / dt_full;
  double *fl = w->nf, *vel = w->nvel, *v_avg = w->nvavg;
  for (int e = 0; e < E; e++)
    for (int m = 0; m < M; m++) {
      fl[e * M + m] = log(f[FIDX(s, k, e, m)]);
      double muval = g->mugrid[m];
      double a = -muval * DuParDt;
      double b = muval * muval * (DlnNDt - DlnBDt) + half * (one - muval * muval) * DlnBDt;
      vel[e * M + m] = cool_damp_fac * (a * g->vgrid_i[e] + b);
      if (fabs(vel[e * M + m]) > vel_abs_max) vel_abs_max = fabs(vel[e * M + m]);
    }
  for (int e = 0; e < E - 1; e++)
    for (int m = 0; m < M; m++)
      v_avg[(e + 1) * M + m] = half * (vel[(e + 1) * M + m] + vel[e * M + m]);
  for (int m = 0; m < M; m++) {
    v_avg[0 * M + m] = v_avg[1 * M + m];
    v_avg[E * M + m] = v_avg[(E - 1) * M + m];
  }
  double dt_stable = safety_factor * g->dlnp / vel_abs_max;
  double nsub = ceil(dt / dt_stable);
  if (!(nsub <= (double)cap))
    return orc_fail(job, EPREM_GPU_ERR_SUBCYCLES, "Adiabatic Change", s, k);
  int N_sub = (int)nsub;
  if (N_sub > job->stats.max_subcycles_change) job->stats.max_subcycles_change = N_sub;
  double dt_sub = dt / N_sub;
  double rmag = NODE(EPREM_NODE_RMAG, s, k);
  orc_opctx_t ctx = {w, p->adiabatic_change_alg, E, M, g->dlnp,
                     log(orc_seed_function(p, g->egrid[0], rmag)),
                     log(orc_seed_function(p, g->egrid[E - 1], rmag)), p, g, rmag};
  orc_subcycle(p->adiabatic_change_alg, N_sub, dt_sub, fl, w->nf1, w->ns1, E * M, orc_change_op, &ctx);
  job->stats.change_cell_subcycles += (double)N_sub * E * M;
  for (int e = 0; e < E; e++)
    for (int m = 0; m < M; m++) {
      double val = exp(fl[e * M + m]);
      f[FIDX(s, k, e, m)] = val;
      if (orc_check(job, val, "Adiabatic Change", s, k)) return job->status;
      if (val < DBL_MIN) f[FIDX(s, k, e, m)] = DBL_MIN;
    }
  return EPREM_GPU_OK;
}

static void orc_work_alloc(orc_work_t *w, int N, int E, int M) {
  size_t nm = (size_t)N * M, em = (size_t)(E + 1) * (M + 1);
  w->list = (int *)malloc(sizeof(int) * N);
  w->ref = (int *)malloc(sizeof(int) * N);
  w->ds_list = (double *)malloc(sizeof(double) * N);
  w->ds_i = (double *)malloc(sizeof(double) * N);
  w->f_old = (double *)malloc(sizeof(double) * nm);
  w->f_new = (double *)malloc(sizeof(double) * nm);
  w->iso = (double *)malloc(sizeof(double) * N);
  w->mult = (double *)malloc(sizeof(double) * N);
  w->emt = (double *)malloc(sizeof(double) * N);
  w->del_fac = (double *)malloc(sizeof(double) * M);
  w->nf = (double *)malloc(sizeof(double) * em);
  w->nf1 = (double *)malloc(sizeof(double) * em);
  w->nvel = (double *)malloc(sizeof(double) * em);
  w->nvavg = (double *)malloc(sizeof(double) * em);
  w->ns1 = (double *)malloc(sizeof(double) * em);
  w->nflux = (double *)malloc(sizeof(double) * em);
  w->nLP = (double *)malloc(sizeof(double) * em);
  w->nLN = (double *)malloc(sizeof(double) * em);
  w->nalpha = (double *)malloc(sizeof(double) * em);
}

static void orc_work_free(orc_work_t *w) {
  free(w->list); free(w->ref); free(w->ds_list); free(w->ds_i); free(w->f_old);
  free(w->f_new); free(w->iso); free(w->mult); free(w->emt); free(w->del_fac);
  free(w->nf); free(w->nf1); free(w->nvel); free(w->nvavg); free(w->ns1);
  free(w->nflux); free(w->nLP); free(w->nLN); free(w->nalpha);
}

/* updateEnergeticParticles (src/energeticParticles.c:70-203) for the streams
 * of one job, sub-steps [step0, step1).  The reference loops sub-steps
 * outermost and, inside each, streams all streams before focusing/changing
 * them; without shell diffusion the streams share no data, so running each
 * stream's sub-steps back to back gives the same values.  With it, the caller
 * runs one sub-step at a time and diffuses across streams in between. */
static void *orc_job_run(void *arg) {
  orc_job_t *job = (orc_job_t *)arg;
  const eprem_dims_t *d = job->d;
  const eprem_params_t *p = job->p;
  const eprem_grids_t *g = job->g;
  const int N = d->num_nodes, E = d->num_energies;
  const size_t SN = (size_t)d->num_streams * N;
  double *nodes = job->nodes;
  orc_work_t w;
  orc_work_alloc(&w, N, E, d->num_mu);
  double dt = p->t_del / (1.0 * p->num_ep_steps);
  for (int s = job->s0; s < job->s1 && job->status == EPREM_GPU_OK; s++) {
    for (int step = job->step0; step < job->step1; step++) {
      orc_stream_values(job, s);
      if (p->check_seed_population > 0) orc_seed_check(job, s);
      if (p->use_parallel_diffusion > 0) {
        double dsMin;
        int L = orc_stream_list(job, &w, s, &dsMin);
        if (L < 0) break;
        if (orc_diffuse_stream(job, &w, s, L, dsMin, dt)) break;
      }
      for (int e = 0; e < E; e++)
        for (int k = 1; k < N; k++) {
          double tau = orc_mfp(p, g, e, NODE(EPREM_NODE_RMAG, s, k), NODE(EPREM_NODE_BMAG, s, k)) *
                       g->vgrid_i[e];
          if (tau < job->stats.min_tau) job->stats.min_tau = tau;
        }
      if (p->use_adiabatic_focus > 0)
        for (int k = 1; k < N; k++)
          if (orc_focus_node(job, &w, s, k, dt)) break;
      if (job->status) break;
      if (p->use_adiabatic_change > 0)
        for (int k = 1; k < N; k++)
          if (orc_change_node(job, &w, s, k, dt)) break;
      if (job->status) break;
    }
  }
  orc_work_free(&w);
  return NULL;
}

static int orc_validate(const eprem_dims_t *d, const eprem_params_t *p, char *errbuf) {
  const char *why = NULL;
  if (d->num_species != 1) why = "num_species must be 1";
  else if (d->num_nodes < 3) why = "num_nodes must be >= 3";
  else if (d->num_energies < 2 || d->num_mu < 2) why = "num_energies and num_mu must be >= 2";
  else if ((p->adiabatic_focus_alg == 3 && d->num_mu < 4) ||
           (p->adiabatic_change_alg == 3 && d->num_energies < 4))
    why = "WENO3 needs at least 4 cells along its axis";
  else if (p->mfp_type != 1 && p->mfp_type != 2) why = "mfp_type must be 1 or 2";
  else if (p->num_ep_steps < 1) why = "num_ep_steps must be >= 1";
  if (why) {
    if (errbuf) snprintf(errbuf, 256, "%s", why);
    return EPREM_GPU_ERR_ARG;
  }
  return EPREM_GPU_OK;
}

/* ShellData (src/energeticParticles.c:254-413): per node and NEWS neighbour,
 * the distance dl to the neighbour's node on the same shell and its part
 * perpendicular to B, dl * sqrt(1 - (e_n . e_B)^2).  dlper: [S][N][4] in the
 * order north, east, west, south. */
static void orc_shell_lengths(const eprem_dims_t *d, const eprem_params_t *p,
                              const double *nodes, const int32_t *news, double *dlper,
                              double *dlen) {
  const int S = d->num_streams, N = d->num_nodes;
  const size_t SN = (size_t)S * N;
  const double rs = p->r_scale;
  for (int s = 0; s < S; s++)
    for (int k = 0; k < N; k++) {
      double rx = NODE(EPREM_NODE_RX, s, k) * rs, ry = NODE(EPREM_NODE_RY, s, k) * rs,
             rz = NODE(EPREM_NODE_RZ, s, k) * rs;
      double bmag = NODE(EPREM_NODE_BMAG, s, k);
      double ebx = NODE(EPREM_NODE_BVEC_X, s, k) / bmag, eby = NODE(EPREM_NODE_BVEC_Y, s, k) / bmag,
             ebz = NODE(EPREM_NODE_BVEC_Z, s, k) / bmag;
      for (int dir = 0; dir < 4; dir++) {
        const int o = news[s * 4 + dir];
        double ex = NODE(EPREM_NODE_RX, o, k) * rs - rx, ey = NODE(EPREM_NODE_RY, o, k) * rs - ry,
               ez = NODE(EPREM_NODE_RZ, o, k) * rs - rz;
        double dl = sqrt(ex * ex + ey * ey + ez * ez);
        dlen[((size_t)s * N + k) * 4 + dir] = dl;
        ex /= dl;
        ey /= dl;
        ez /= dl;
        double dot = ex * ebx + ey * eby + ez * ebz;
        dlper[((size_t)s * N + k) * 4 + dir] = dl * sqrt(1.0 - dot * dot);
      }
    }
}

/* DiffuseShellData (src/energeticParticles.c:419-554), one sub-step of
 * length dt over all streams, nodes 1..N-1 (shells innerComputeShell on):
 * per node and energy, each stream hands delta = min(dt kper / dlPer^2,
 * 0.025) of its f to each NEWS neighbour, kper = dt * 0.33333333 * mfp * v
 * * kperxkpar as the reference writes it; all deltas of one node and energy
 * are summed (in the reference's order: source streams ascending, north,
 * east, west, south, then the source's own loss) before f changes. */
static int orc_shell_diffuse(const eprem_dims_t *d, const eprem_params_t *p,
                             const eprem_grids_t *g, double *f, const double *nodes,
                             const int32_t *news, double kperxkpar, const double *dlper,
                             double dt, char *errbuf) {
  const int S = d->num_streams, N = d->num_nodes, E = d->num_energies, M = d->num_mu;
  const size_t SN = (size_t)S * N;
  const double thresh = 0.025, verysmall = 1.0e-33;
  double *delta = (double *)malloc(sizeof(double) * (size_t)S * M);
  int rc = EPREM_GPU_OK;
  for (int k = 1; k < N && !rc; k++)
    for (int e = 0; e < E && !rc; e++) {
      for (size_t i = 0; i < (size_t)S * M; i++) delta[i] = 0.0;
      for (int s = 0; s < S; s++) {
        double mfp = orc_mfp(p, g, e, NODE(EPREM_NODE_RMAG, s, k), NODE(EPREM_NODE_BMAG, s, k));
        double dt_kper = dt * 0.33333333 * mfp * g->vgrid[e] * kperxkpar;
        double del[4];
        for (int dir = 0; dir < 4; dir++) {
          double l = dlper[((size_t)s * N + k) * 4 + dir];
          del[dir] = dt_kper / (l * l + verysmall);
          if (del[dir] > thresh) del[dir] = thresh;
        }
        const double *fs = &f[FIDX(s, k, e, 0)];
        for (int m = 0; m < M; m++) {
          for (int dir = 0; dir < 4; dir++) delta[(size_t)news[s * 4 + dir] * M + m] += del[dir] * fs[m];
          delta[(size_t)s * M + m] -= (del[0] + del[1] + del[2] + del[3]) * fs[m];
        }
      }
      for (int s = 0; s < S && !rc; s++)
        for (int m = 0; m < M; m++) {
          double v = f[FIDX(s, k, e, m)] += delta[(size_t)s * M + m];
          if (isnan(v) || isinf(v)) {
            rc = isnan(v) ? EPREM_GPU_ERR_NAN : EPREM_GPU_ERR_INF;
            if (errbuf)
              snprintf(errbuf, 256, "%s in DiffuseShellData (stream %d, node %d)",
                       isnan(v) ? "NaN value" : "Inf value", s, k);
            break;
          }
        }
    }
  free(delta);
  return rc;
}

/* driftVelocity (src/energeticParticles.c:210-246) for energy e: the
 * spherical curl(B)/B^2 times (1/om1) p v / 3, p = exp(lnpmin + e dlnp),
 * om1 = charge OM / mass, to Cartesian at position r (sphToCartVector,
 * src/geometry.c:89-125). */
#define ORC_Q 4.80320425e-10
#define ORC_OM (ORC_MHD_B_NORM * ORC_Q * ORC_AU / (ORC_MP * ORC_C * ORC_C))
static void orc_drift_velocity(const eprem_drift_params_t *dp, const eprem_grids_t *g, int e,
                               const double curl[3], double x, double y, double z,
                               double out[3]) {
  double pm = exp(dp->lnpmin + e * g->dlnp);
  double om1 = dp->charge * ORC_OM / dp->mass;
  double factor = (1.0 / om1) * (pm * g->vgrid[e] / 3.0);
  double vr = factor * curl[0], vt = factor * curl[1], vp = factor * curl[2];
  double rmag = sqrt(x * x + y * y + z * z);
  if ((rmag - fabs(z)) < ORC_VERYSMALL) {
    out[0] = 0.0;
    out[1] = 0.0;
  } else {
    out[0] = x / rmag * vr + x * z / (rmag * sqrt(rmag * rmag - z * z)) * vt -
             y / sqrt(rmag * rmag - z * z) * vp;
    out[1] = y / rmag * vr + y * z / (rmag * sqrt(rmag * rmag - z * z)) * vt +
             x / sqrt(rmag * rmag - z * z) * vp;
  }
  out[2] = z / rmag * vr - sqrt(rmag * rmag - z * z) / rmag * vt;
}

/* DriftShellData (src/energeticParticles.c:561-801), one sub-step of length
 * dt over all streams, nodes 1..N-1: per node and energy, each stream hands
 * del = min(vdp dt / dl, THRESH) of its f to every NEWS neighbour with
 * vdp = (v_d . (r_nbr - r)) rScale / dl > 0 (dl the neighbour distance of
 * ShellData), all hand-overs of one node and energy summed in the
 * reference's order (source streams ascending; per source north, east, west,
 * south, each with its gain to the neighbour and then the source's loss)
 * before f changes. */
static int orc_drift_shell(const eprem_dims_t *d, const eprem_params_t *p,
                           const eprem_grids_t *g, double *f, const double *nodes,
                           const int32_t *news, const double *dlen, const double *curl,
                           const eprem_drift_params_t *dp, double dt, char *errbuf) {
  const int S = d->num_streams, N = d->num_nodes, E = d->num_energies, M = d->num_mu;
  const size_t SN = (size_t)S * N;
  const double thresh = 0.025;
  double *delta = (double *)malloc(sizeof(double) * (size_t)S * M);
  int rc = EPREM_GPU_OK;
  for (int k = 1; k < N && !rc; k++)
    for (int e = 0; e < E && !rc; e++) {
      for (size_t i = 0; i < (size_t)S * M; i++) delta[i] = 0.0;
      for (int s = 0; s < S; s++) {
        const double x = NODE(EPREM_NODE_RX, s, k), y = NODE(EPREM_NODE_RY, s, k),
                     z = NODE(EPREM_NODE_RZ, s, k);
        const double cv[3] = {curl[0 * SN + (size_t)s * N + k], curl[1 * SN + (size_t)s * N + k],
                              curl[2 * SN + (size_t)s * N + k]};
        double vd[3];
        orc_drift_velocity(dp, g, e, cv, x, y, z, vd);
        const double *fs = &f[FIDX(s, k, e, 0)];
        for (int dir = 0; dir < 4; dir++) {
          const int o = news[s * 4 + dir];
          double enx = NODE(EPREM_NODE_RX, o, k) - x, eny = NODE(EPREM_NODE_RY, o, k) - y,
                 enz = NODE(EPREM_NODE_RZ, o, k) - z;
          const double dl = dlen[((size_t)s * N + k) * 4 + dir];
          double vdp = (vd[0] * enx + vd[1] * eny + vd[2] * enz) * p->r_scale / dl;
          if (vdp > 0.0) {
            double del = vdp * dt / dl;
            if (del > thresh) del = thresh;
            for (int m = 0; m < M; m++) {
              delta[(size_t)o * M + m] += del * fs[m];
              delta[(size_t)s * M + m] -= del * fs[m];
            }
          }
        }
      }
      for (int s = 0; s < S && !rc; s++)
        for (int m = 0; m < M; m++) {
          double v = f[FIDX(s, k, e, m)] += delta[(size_t)s * M + m];
          if (isnan(v) || isinf(v)) {
            rc = isnan(v) ? EPREM_GPU_ERR_NAN : EPREM_GPU_ERR_INF;
            if (errbuf)
              snprintf(errbuf, 256, "%s in DriftShellData (stream %d, node %d)",
                       isnan(v) ? "NaN value" : "Inf value", s, k);
            break;
          }
        }
    }
  free(delta);
  return rc;
}

static int orc_update_core(const eprem_dims_t *d, const eprem_params_t *p, const eprem_grids_t *g,
                           double *f, double *nodes, int s0, int s1, const int32_t *news,
                           int shell_on, double kperxkpar, const eprem_drift_params_t *drift,
                           const double *curl, eprem_ep_stats_t *stats, int nthreads,
                           char *errbuf) {
  int rc = orc_validate(d, p, errbuf);
  if (rc) return rc;
  if (s0 < 0) s0 = 0;
  if (s1 > d->num_streams) s1 = d->num_streams;
  int ns = s1 - s0;
  if (ns <= 0) return EPREM_GPU_OK;
  if (news) {
    if (ns != d->num_streams) {
      if (errbuf) snprintf(errbuf, 256, "shell diffusion couples all streams: no stream range");
      return EPREM_GPU_ERR_ARG;
    }
    for (int i = 0; i < 4 * d->num_streams; i++)
      if (news[i] < 0 || news[i] >= d->num_streams) {
        if (errbuf) snprintf(errbuf, 256, "NEWS neighbour out of range");
        return EPREM_GPU_ERR_ARG;
      }
  }
  if (nthreads < 1) nthreads = 1;
  if (nthreads > ns) nthreads = ns;
  orc_job_t *jobs = (orc_job_t *)calloc(nthreads, sizeof(orc_job_t));
  pthread_t *th = (pthread_t *)calloc(nthreads, sizeof(pthread_t));
  for (int t = 0; t < nthreads; t++) {
    jobs[t].d = d; jobs[t].p = p; jobs[t].g = g; jobs[t].f = f; jobs[t].nodes = nodes;
    jobs[t].s0 = s0 + (int)((long)ns * t / nthreads);
    jobs[t].s1 = s0 + (int)((long)ns * (t + 1) / nthreads);
    jobs[t].stats.min_tau = DBL_MAX;
    jobs[t].status = EPREM_GPU_OK;
  }
  /* Without shell diffusion one pass runs every sub-step; with it, one pass
   * per sub-step, each followed by the diffusion over all streams. */
  const int passes = news ? p->num_ep_steps : 1;
  double *dlper = NULL, *dlen = NULL;
  if (news) {
    dlper = (double *)malloc(sizeof(double) * 4 * (size_t)d->num_streams * d->num_nodes);
    dlen = (double *)malloc(sizeof(double) * 4 * (size_t)d->num_streams * d->num_nodes);
    orc_shell_lengths(d, p, nodes, news, dlper, dlen);
  }
  const double dt = p->t_del / (1.0 * p->num_ep_steps);
  int diff_rc = EPREM_GPU_OK;
  char diff_err[256] = "";
  for (int pass = 0; pass < passes && !diff_rc; pass++) {
    for (int t = 0; t < nthreads; t++) {
      jobs[t].step0 = news ? pass : 0;
      jobs[t].step1 = news ? pass + 1 : p->num_ep_steps;
    }
    if (nthreads == 1) {
      orc_job_run(&jobs[0]);
    } else {
      for (int t = 0; t < nthreads; t++) pthread_create(&th[t], NULL, orc_job_run, &jobs[t]);
      for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
    }
    int failed = 0;
    for (int t = 0; t < nthreads; t++) failed |= jobs[t].status != EPREM_GPU_OK;
    if (failed) break;
    if (news && shell_on)
      diff_rc = orc_shell_diffuse(d, p, g, f, nodes, news, kperxkpar, dlper, dt, diff_err);
    if (news && drift && !diff_rc)
      diff_rc = orc_drift_shell(d, p, g, f, nodes, news, dlen, curl, drift, dt, diff_err);
  }
  free(dlper);
  free(dlen);
  rc = EPREM_GPU_OK;
  for (int t = 0; t < nthreads; t++) {
    eprem_ep_stats_t *js = &jobs[t].stats;
    if (js->max_subcycles_change > stats->max_subcycles_change)
      stats->max_subcycles_change = js->max_subcycles_change;
    if (js->max_subcycles_focusing > stats->max_subcycles_focusing)
      stats->max_subcycles_focusing = js->max_subcycles_focusing;
    if (js->max_substeps_stream > stats->max_substeps_stream)
      stats->max_substeps_stream = js->max_substeps_stream;
    if (js->min_tau < stats->min_tau) stats->min_tau = js->min_tau;
    stats->stream_cell_subcycles += js->stream_cell_subcycles;
    stats->focus_cell_subcycles += js->focus_cell_subcycles;
    stats->change_cell_subcycles += js->change_cell_subcycles;
    if (rc == EPREM_GPU_OK && jobs[t].status != EPREM_GPU_OK) {
      rc = jobs[t].status;
      if (errbuf) snprintf(errbuf, 256, "%s", jobs[t].err);
    }
  }
  if (rc == EPREM_GPU_OK && diff_rc != EPREM_GPU_OK) {
    rc = diff_rc;
    if (errbuf) snprintf(errbuf, 256, "%s", diff_err);
  }
  free(jobs);
  free(th);
  return rc;
}

int orc_update_energetic_particles_range(const eprem_dims_t *d, const eprem_params_t *p,
                                         const eprem_grids_t *g, double *f, double *nodes,
                                         int s0, int s1, eprem_ep_stats_t *stats, int nthreads,
                                         char *errbuf) {
  return orc_update_core(d, p, g, f, nodes, s0, s1, NULL, 0, 0.0, NULL, NULL, stats, nthreads,
                         errbuf);
}

int orc_update_energetic_particles_news(const eprem_dims_t *d, const eprem_params_t *p,
                                        const eprem_grids_t *g, double *f, double *nodes,
                                        const int32_t *news, double kperxkpar,
                                        eprem_ep_stats_t *stats, int nthreads, char *errbuf) {
  return orc_update_core(d, p, g, f, nodes, 0, d->num_streams, news, 1, kperxkpar, NULL, NULL,
                         stats, nthreads, errbuf);
}

int orc_update_energetic_particles_perp(const eprem_dims_t *d, const eprem_params_t *p,
                                        const eprem_grids_t *g, double *f, double *nodes,
                                        const int32_t *news, int shell_on, double kperxkpar,
                                        const eprem_drift_params_t *drift, const double *curl,
                                        eprem_ep_stats_t *stats, int nthreads, char *errbuf) {
  if (drift && !curl) {
    if (errbuf) snprintf(errbuf, 256, "drift needs curl(B)/B^2");
    return EPREM_GPU_ERR_ARG;
  }
  return orc_update_core(d, p, g, f, nodes, 0, d->num_streams, news, shell_on, kperxkpar, drift,
                         curl, stats, nthreads, errbuf);
}

int orc_update_energetic_particles(const eprem_dims_t *d, const eprem_params_t *p,
                                   const eprem_grids_t *g, double *f, double *nodes,
                                   eprem_ep_stats_t *stats, int nthreads, char *errbuf) {
  return orc_update_energetic_particles_range(d, p, g, f, nodes, 0, d->num_streams, stats,
                                              nthreads, errbuf);
}

/* ------------------------------------------------------------------------ */
/* idealShockFactor, src/flow.c:623-651. */
static double orc_shock_factor(const eprem_params_t *p, double r, double t_global) {
  double exponent = exp(2.0 * (p->ideal_shock_sharpness / p->ideal_shock_scale_length) *
                        (r - ((p->ideal_shock_speed / ORC_C) *
                                  (t_global - p->ideal_shock_init_time / ORC_DAY) +
                              p->r_scale)));
  double ratio;
  if (exponent >= 1.0e8)
    ratio = 1.0;
  else if (exponent <= 1.0e-8)
    ratio = -1.0;
  else
    ratio = (exponent - 1.0) / (exponent + 1.0);
  double factor = (1.0 + ((1.0 - ratio) * 0.5 * (p->ideal_shock_jump - 1.0)));
  double falloff = exp(p->ideal_shock_falloff *
                       (r - ((p->ideal_shock_speed / ORC_C) *
                                 (t_global - p->ideal_shock_init_time / ORC_DAY) +
                             p->r_scale)));
  return 1 + (factor - 1) * falloff;
}

/* parkerB (src/flow.c:443-472) at (r AU, theta), ideal shock included. */
static void orc_parker_b(const eprem_params_t *p, double r, double theta, double Vr, int isn,
                         double t_global, double B[3]) {
  B[0] = p->mhd_bs_au / (r * r);
  B[1] = 0.0;
  B[2] = -1.0 * r * B[0] * (p->omega_sun / (Vr + ORC_VERYSMALL)) * sin(theta);
  if ((p->ideal_shock > 0) && (isn > 0)) {
    B[0] *= orc_shock_factor(p, r, t_global);
    B[1] *= orc_shock_factor(p, r, t_global);
    B[2] *= orc_shock_factor(p, r, t_global);
  }
}

/* curlBoverB2 (src/flow.c:479-616): curl(B)/B^2 of the Parker field by
 * centred differences at (r +- 0.001 AU, theta +- pi/100, phi +- pi/100),
 * angles folded back into range; spherical components (r, theta, phi). */
static void orc_curl_bover_b2(const eprem_params_t *p, double x, double y, double z, double Vr,
                              int isn, double t_global, double curl[3]) {
  const double rcw = 0.001, tcw = ORC_PI / 100.0, pcw = ORC_PI / 100.0;
  double rr = p->r_scale * sqrt(x * x + y * y + z * z);
  double th = acos(z * p->r_scale / rr);
  double ph = atan2(y, x);
  double rp = rr + rcw, rm = rr - rcw;
  double tp = th + tcw, tp_ph = ph;
  if (tp > ORC_PI) {
    tp = 2.0 * ORC_PI - tp;
    tp_ph += ORC_PI;
    if (tp_ph > (2.0 * ORC_PI)) tp_ph -= (2.0 * ORC_PI);
  }
  double tm = th - tcw, tm_ph = ph;
  if (tm < 0.0) {
    tm *= -1.0;
    tm_ph += ORC_PI;
    if (tm_ph > (2.0 * ORC_PI)) tm_ph -= (2.0 * ORC_PI);
  }
  (void)tp_ph;
  (void)tm_ph;  /* parkerB depends on r and theta only */
  double B_rm[3], B_rp[3], B_tm[3], B_tp[3], B_pm[3], B_pp[3];
  orc_parker_b(p, rm, th, Vr, isn, t_global, B_rm);
  orc_parker_b(p, rp, th, Vr, isn, t_global, B_rp);
  orc_parker_b(p, rr, tm, Vr, isn, t_global, B_tm);
  orc_parker_b(p, rr, tp, Vr, isn, t_global, B_tp);
  orc_parker_b(p, rr, th, Vr, isn, t_global, B_pm);
  orc_parker_b(p, rr, th, Vr, isn, t_global, B_pp);
  double m_rm = sqrt(B_rm[0] * B_rm[0] + B_rm[1] * B_rm[1] + B_rm[2] * B_rm[2]);
  double m_rp = sqrt(B_rp[0] * B_rp[0] + B_rp[1] * B_rp[1] + B_rp[2] * B_rp[2]);
  double m_tm = sqrt(B_tm[0] * B_tm[0] + B_tm[1] * B_tm[1] + B_tm[2] * B_tm[2]);
  double m_tp = sqrt(B_tp[0] * B_tp[0] + B_tp[1] * B_tp[1] + B_tp[2] * B_tp[2]);
  double m_pm = sqrt(B_pm[0] * B_pm[0] + B_pm[1] * B_pm[1] + B_pm[2] * B_pm[2]);
  double m_pp = sqrt(B_pp[0] * B_pp[0] + B_pp[1] * B_pp[1] + B_pp[2] * B_pp[2]);
  double A, B;
  A = (0.5 / tcw) * (B_tp[2] * sin(tp) / (m_tp * m_tp) - B_tm[2] * sin(tm) / (m_tm * m_tm));
  B = (0.5 / pcw) * (B_pp[1] / (m_pp * m_pp) - B_pm[1] / (m_pm * m_pm));
  curl[0] = (1.0 / (rr * sin(th))) * (A - B);
  A = (1.0 / sin(th)) * (0.5 / pcw) * (B_pp[0] / (m_pp * m_pp) - B_pm[0] / (m_pm * m_pm));
  B = (0.5 / rcw) * (rp * B_rp[2] / (m_rp * m_rp) - rm * B_rm[2] / (m_rm * m_rm));
  curl[1] = (1.0 / rr) * (A - B);
  A = (0.5 / rcw) * (rp * B_rp[1] / (m_rp * m_rp) - rm * B_rm[1] / (m_rm * m_rm));
  B = (0.5 / tcw) * (B_tp[0] / (m_tp * m_tp) - B_tm[0] / (m_tm * m_tm));
  curl[2] = (1.0 / rr) * (A - B);
}

static int orc_update_mhd_core(const eprem_dims_t *d, const eprem_params_t *p, double *nodes,
                               double t_global, double *curl);

/* updateMhd with mhdGridStatus == MHD_DEFAULT (src/flow.c:36-154), including
 * mhdDensity (:241-275), mhdV (:356-403), mhdB (:281-350). */
int orc_update_mhd(const eprem_dims_t *d, const eprem_params_t *p, double *nodes,
                   double t_global) {
  return orc_update_mhd_core(d, p, nodes, t_global, NULL);
}

/* The same with useDrift on: curl(B)/B^2 of every node (mhdCurlBoverB2,
 * src/flow.c:127-128) into curl[3][S*N] (r, theta, phi). */
int orc_update_mhd_curl(const eprem_dims_t *d, const eprem_params_t *p, double *nodes,
                        double t_global, double *curl) {
  return orc_update_mhd_core(d, p, nodes, t_global, curl);
}

static int orc_update_mhd_core(const eprem_dims_t *d, const eprem_params_t *p, double *nodes,
                               double t_global, double *curl) {
  const int N = d->num_nodes;
  const size_t SN = (size_t)d->num_streams * N;
  const double rs = p->r_scale;
  for (int s = 0; s < d->num_streams; s++)
    for (int k = 0; k < N; k++) {
      NODE(EPREM_NODE_BMAG_OLD, s, k) = NODE(EPREM_NODE_BMAG, s, k);
      NODE(EPREM_NODE_DENSITY_OLD, s, k) = NODE(EPREM_NODE_DENSITY, s, k);
      NODE(EPREM_NODE_VSPH_OLD_R, s, k) = NODE(EPREM_NODE_VR, s, k);
      NODE(EPREM_NODE_VSPH_OLD_THETA, s, k) = NODE(EPREM_NODE_VTHETA, s, k);
      NODE(EPREM_NODE_VSPH_OLD_PHI, s, k) = NODE(EPREM_NODE_VPHI, s, k);
      NODE(EPREM_NODE_DS_OLD, s, k) = NODE(EPREM_NODE_DS, s, k);
      NODE(EPREM_NODE_ROLDER_X, s, k) = NODE(EPREM_NODE_RX, s, k);
      NODE(EPREM_NODE_ROLDER_Y, s, k) = NODE(EPREM_NODE_RY, s, k);
      NODE(EPREM_NODE_ROLDER_Z, s, k) = NODE(EPREM_NODE_RZ, s, k);
      double x = NODE(EPREM_NODE_RX, s, k), y = NODE(EPREM_NODE_RY, s, k),
             z = NODE(EPREM_NODE_RZ, s, k), rmag = NODE(EPREM_NODE_RMAG, s, k);
      int isn = 0;
      if (p->ideal_shock > 0) {
        /* cartToSphPosAu, src/geometry.c:131-150 */
        double ax = x * rs, ay = y * rs, az = z * rs;
        double rr = sqrt(ax * ax + ay * ay + az * az);
        double th = acos(az / rr);
        double ph = atan2(ay, ax);
        while (ph < 0.0) ph += (2.0 * ORC_PI);
        if (rr <= p->ideal_shock_speed * t_global) {
          if (p->ideal_shock_width == 0.0)
            isn = 1;
          else if ((fmin((2 * ORC_PI) - fabs(ph - p->ideal_shock_phi), fabs(ph - p->ideal_shock_phi)) <
                    (p->ideal_shock_width / (double)2.0)) &&
                   (fabs(th - p->ideal_shock_theta) < (p->ideal_shock_width / 2.0)))
            isn = 1;
        }
      }
      double rr = rmag * rs;
      double dens = p->mhd_ns_au / (rr * rr);
      if ((p->ideal_shock > 0) && (isn > 0)) dens *= orc_shock_factor(p, rr, t_global);
      NODE(EPREM_NODE_DENSITY, s, k) = dens;
      if (dens <= 0.0)
        NODE(EPREM_NODE_DIVV, s, k) = 0.0;
      else
        NODE(EPREM_NODE_DIVV, s, k) = -1.0 * log(dens / NODE(EPREM_NODE_DENSITY_OLD, s, k)) / p->t_del;
      double theta = acos(z / rmag);
      double phi = atan2(y, x);
      double Vr = p->mhd_us;
      if ((p->ideal_shock > 0) && (isn > 0)) Vr *= orc_shock_factor(p, rmag * rs, t_global);
      double Vt = 0.0, Vp = 0.0;
      NODE(EPREM_NODE_VR, s, k) = Vr;
      NODE(EPREM_NODE_VTHETA, s, k) = Vt;
      NODE(EPREM_NODE_VPHI, s, k) = Vp;
      NODE(EPREM_NODE_VMAG, s, k) = sqrt(Vr * Vr + Vt * Vt + Vp * Vp);
      NODE(EPREM_NODE_VVEC_X, s, k) = Vr * sin(theta) * cos(phi) + Vt * cos(theta) * cos(phi) - Vp * sin(phi);
      NODE(EPREM_NODE_VVEC_Y, s, k) = Vr * sin(theta) * sin(phi) + Vt * cos(theta) * sin(phi) + Vp * cos(phi);
      NODE(EPREM_NODE_VVEC_Z, s, k) = Vr * cos(theta) - Vt * sin(theta);
      double Br = p->mhd_bs_au / (rr * rr);
      double Bt = 0.0;
      double Bp = -1.0 * rr * Br * (p->omega_sun / (Vr + ORC_VERYSMALL)) * sin(theta);
      NODE(EPREM_NODE_BR, s, k) = Br;
      NODE(EPREM_NODE_BTHETA, s, k) = Bt;
      NODE(EPREM_NODE_BPHI, s, k) = Bp;
      double Bmag = sqrt(Br * Br + Bt * Bt + Bp * Bp);
      NODE(EPREM_NODE_BMAG, s, k) = Bmag;
      NODE(EPREM_NODE_BVEC_X, s, k) = Br * sin(theta) * cos(phi) + Bt * cos(theta) * cos(phi) - Bp * sin(phi);
      NODE(EPREM_NODE_BVEC_Y, s, k) = Br * sin(theta) * sin(phi) + Bt * cos(theta) * sin(phi) + Bp * cos(phi);
      NODE(EPREM_NODE_BVEC_Z, s, k) = Br * cos(theta) - Bt * sin(theta);
      if (curl) {
        double cv[3];
        orc_curl_bover_b2(p, x, y, z, Vr, isn, t_global, cv);
        for (int c = 0; c < 3; c++) curl[(size_t)c * SN + (size_t)s * N + k] = cv[c];
      }
      if (k == 0) {
        NODE(EPREM_NODE_DUPAR, s, k) = 0.0;
        NODE(EPREM_NODE_DLNB, s, k) = 0.0;
        NODE(EPREM_NODE_DLNN, s, k) = 0.0;
      } else {
        double dupar = (Vr - NODE(EPREM_NODE_VSPH_OLD_R, s, k)) * Br +
                       (Vt - NODE(EPREM_NODE_VSPH_OLD_THETA, s, k)) * Bt +
                       (Vp - NODE(EPREM_NODE_VSPH_OLD_PHI, s, k)) * Bp;
        dupar /= Bmag;
        NODE(EPREM_NODE_DUPAR, s, k) = dupar;
        NODE(EPREM_NODE_DLNB, s, k) = log(Bmag / NODE(EPREM_NODE_BMAG_OLD, s, k));
        NODE(EPREM_NODE_DLNN, s, k) = log(dens / NODE(EPREM_NODE_DENSITY_OLD, s, k));
      }
    }
  return EPREM_GPU_OK;
}

/* moveNodes, src/simCore.c:737-785 (MHD_DEFAULT branch of delrFlow). */
int orc_move_nodes(const eprem_dims_t *d, const eprem_params_t *p, double *nodes, double dt) {
  const int N = d->num_nodes;
  const size_t SN = (size_t)d->num_streams * N;
  for (int s = 0; s < d->num_streams; s++)
    for (int k = 1; k < N; k++) {
      double x = NODE(EPREM_NODE_RX, s, k), y = NODE(EPREM_NODE_RY, s, k), z = NODE(EPREM_NODE_RZ, s, k);
      double dx = dt * NODE(EPREM_NODE_VVEC_X, s, k) / p->r_scale;
      double dy = dt * NODE(EPREM_NODE_VVEC_Y, s, k) / p->r_scale;
      double dz = dt * NODE(EPREM_NODE_VVEC_Z, s, k) / p->r_scale;
      NODE(EPREM_NODE_ROLD_X, s, k) = x;
      NODE(EPREM_NODE_ROLD_Y, s, k) = y;
      NODE(EPREM_NODE_ROLD_Z, s, k) = z;
      x += dx;
      y += dy;
      z += dz;
      NODE(EPREM_NODE_RX, s, k) = x;
      NODE(EPREM_NODE_RY, s, k) = y;
      NODE(EPREM_NODE_RZ, s, k) = z;
      NODE(EPREM_NODE_RMAG, s, k) = sqrt((x * x) + (y * y) + (z * z));
    }
  return EPREM_GPU_OK;
}

/* computeFlux without the output unit scale, src/unifiedOutput.c:153-180. */
void orc_omni_flux(const eprem_dims_t *d, const eprem_grids_t *g, const double *f, double *out) {
  const int N = d->num_nodes, E = d->num_energies, M = d->num_mu;
  for (int s = 0; s < d->num_streams; s++)
    for (int k = 0; k < N; k++)
      for (int e = 0; e < E; e++) {
        double iso = 0.0;
        for (int m = 0; m < M; m++) iso += f[FIDX(s, k, e, m)];
        iso /= M;
        out[((size_t)s * N + k) * E + e] = 2.0 * g->egrid[e] * iso;
      }
}

/* ------------------------------------------------------------------------ */
/* Layout of the public structs as this C compiler lays them out, so the test
 * suite can check the Python (ctypes) mirror field by field. */
#include <stddef.h>
int orc_abi_layout(long *out, int cap) {
  int n = 0;
#define PUT(x) do { if (n < cap) out[n] = (long)(x); n++; } while (0)
  PUT(sizeof(eprem_dims_t));
  PUT(sizeof(eprem_params_t));
  PUT(sizeof(eprem_grids_t));
  PUT(sizeof(eprem_ep_stats_t));
  PUT(EPREM_NODE_NFIELDS);
#define OFF(T, f) PUT(offsetof(T, f))
  OFF(eprem_dims_t, num_streams); OFF(eprem_dims_t, num_nodes); OFF(eprem_dims_t, num_species);
  OFF(eprem_dims_t, num_energies); OFF(eprem_dims_t, num_mu); OFF(eprem_dims_t, precision);
  OFF(eprem_params_t, r_scale); OFF(eprem_params_t, t_del); OFF(eprem_params_t, num_ep_steps);
  OFF(eprem_params_t, use_parallel_diffusion); OFF(eprem_params_t, use_adiabatic_focus);
  OFF(eprem_params_t, use_adiabatic_change); OFF(eprem_params_t, check_seed_population);
  OFF(eprem_params_t, use_ep_boundary); OFF(eprem_params_t, use_boundary_function);
  OFF(eprem_params_t, adiabatic_focus_alg); OFF(eprem_params_t, adiabatic_change_alg);
  OFF(eprem_params_t, damp_cooling); OFF(eprem_params_t, dsh_min); OFF(eprem_params_t, mfp_type);
  OFF(eprem_params_t, lamo); OFF(eprem_params_t, mfp_radial_power); OFF(eprem_params_t, mfp_b_power);
  OFF(eprem_params_t, mhd_bs_au); OFF(eprem_params_t, bf_amplitude); OFF(eprem_params_t, bf_xi);
  OFF(eprem_params_t, bf_gamma); OFF(eprem_params_t, bf_beta); OFF(eprem_params_t, bf_ecutoff);
  OFF(eprem_params_t, bf_r0); OFF(eprem_params_t, mhd_us); OFF(eprem_params_t, mhd_ns_au);
  OFF(eprem_params_t, omega_sun); OFF(eprem_params_t, ideal_shock);
  OFF(eprem_params_t, ideal_shock_sharpness); OFF(eprem_params_t, ideal_shock_scale_length);
  OFF(eprem_params_t, ideal_shock_jump); OFF(eprem_params_t, ideal_shock_falloff);
  OFF(eprem_params_t, ideal_shock_speed); OFF(eprem_params_t, ideal_shock_init_time);
  OFF(eprem_params_t, ideal_shock_theta); OFF(eprem_params_t, ideal_shock_phi);
  OFF(eprem_params_t, ideal_shock_width); OFF(eprem_params_t, max_subcycles);
  OFF(eprem_params_t, stream_variant);
  OFF(eprem_grids_t, egrid); OFF(eprem_grids_t, vgrid); OFF(eprem_grids_t, vgrid_i);
  OFF(eprem_grids_t, mugrid); OFF(eprem_grids_t, rigidity); OFF(eprem_grids_t, dlnp);
  OFF(eprem_grids_t, dmu);
  OFF(eprem_ep_stats_t, max_subcycles_change); OFF(eprem_ep_stats_t, max_subcycles_focusing);
  OFF(eprem_ep_stats_t, max_substeps_stream); OFF(eprem_ep_stats_t, pad);
  OFF(eprem_ep_stats_t, min_tau); OFF(eprem_ep_stats_t, stream_cell_subcycles);
  OFF(eprem_ep_stats_t, focus_cell_subcycles); OFF(eprem_ep_stats_t, change_cell_subcycles);
#undef OFF
#undef PUT
  return n;
}

/* ======================================================================== */
/* MAS coupling.  Unit conversions of src/baseTypes.h:104-115; note that
 * MAS_B_CONVERT expands without parentheses where the reference multiplies by
 * it, so the product is ((((x*sqrt(4 pi rho_n))*L_n)/T_n)/B_norm). */
#define ORC_RSUN 6.96e10
#define ORC_RSAU (ORC_RSUN / ORC_AU)
#define ORC_MAS_LENGTH_NORM 6.96e10
#define ORC_MAS_RHO_NORM 1.6726e-16

typedef struct {
  double br, bt, bp, vr, vt, vp, d;
} orc_masnode_t;

/* masTriLinearBinarySearch, src/masInterp.c:118-171 */
static double orc_mas_search(const float *A, double key, int *imin, int *imax, int lower,
                             int upper) {
  while (upper != (lower + 1)) {
    int imid = (lower + upper) / 2;
    if (A[imid] < key)
      lower = imid;
    else
      upper = imid;
  }
  *imin = lower;
  *imax = upper;
  if (A[*imin] > key) return 0.0;
  if (A[*imax] < key) return 1.0;
  return ((key - A[lower]) / (A[upper] - A[lower]));
}

/* masInterpolate, src/masInterp.c:178-200 */
static double orc_mas_interp(const float *V, int r0, int r1, int t0, int t1, int p0, int p1,
                             double rd, double td, double pd, int rDim, int tDim) {
#define VIX(r, t, p) ((size_t)(r) + (size_t)rDim * (t) + (size_t)rDim * tDim * (p))
  double c00 = V[VIX(r0, t0, p0)] * (1.0 - rd) + V[VIX(r1, t0, p0)] * rd;
  double c10 = V[VIX(r0, t0, p1)] * (1.0 - rd) + V[VIX(r1, t0, p1)] * rd;
  double c01 = V[VIX(r0, t1, p0)] * (1.0 - rd) + V[VIX(r1, t1, p0)] * rd;
  double c11 = V[VIX(r0, t1, p1)] * (1.0 - rd) + V[VIX(r1, t1, p1)] * rd;
#undef VIX
  double c0 = c00 * (1.0 - pd) + c10 * pd;
  double c1 = c01 * (1.0 - pd) + c11 * pd;
  return (c0 * (1.0 - td) + c1 * td);
}

/* One field of masTriLinear: search both slots' meshes and blend in time. */
static double orc_mas_field(const orc_mas_t *mas, int f, double rr, double th, double ph) {
  double val[2];
  for (int sl = 0; sl < 2; sl++) {
    const eprem_mas_slice_t *S = sl ? mas->slot1 : mas->slot0;
    int r0, r1, t0, t1, p0, p1;
    double rd = orc_mas_search(S->mesh[f][0], rr, &r0, &r1, 0, S->dims[f][0] - 1);
    double td = orc_mas_search(S->mesh[f][1], th, &t0, &t1, 0, S->dims[f][1] - 1);
    double pd = orc_mas_search(S->mesh[f][2], ph, &p0, &p1, 0, S->dims[f][2] - 1);
    val[sl] = orc_mas_interp(S->data[f], r0, r1, t0, t1, p0, p1, rd, td, pd, S->dims[f][0],
                             S->dims[f][1]);
  }
  return ((1.0 - mas->s_cor) * val[0] + mas->s_cor * val[1]);
}

/* masTriLinear, src/masInterp.c:539-740 (position: r in AU, theta, phi). */
static void orc_mas_trilinear(const orc_mas_t *mas, double pr, double pth, double pph,
                              orc_masnode_t *out) {
  double rr = pr / ORC_RSAU;
  double th = pth;
  double ph = pph - mas->phi_offset;
  if (ph < 0.0)
    while (ph < 0.0) ph += (2.0 * ORC_PI);
  if (ph > (2.0 * ORC_PI))
    while (ph > (2.0 * ORC_PI)) ph -= (2.0 * ORC_PI);
  double b;
  b = orc_mas_field(mas, 0, rr, th, ph);
  out->bp = b * sqrt(4.0 * ORC_PI * ORC_MAS_RHO_NORM) * ORC_MAS_LENGTH_NORM / ORC_MAS_TIME_NORM / ORC_MHD_B_NORM;
  b = orc_mas_field(mas, 1, rr, th, ph);
  out->bt = b * sqrt(4.0 * ORC_PI * ORC_MAS_RHO_NORM) * ORC_MAS_LENGTH_NORM / ORC_MAS_TIME_NORM / ORC_MHD_B_NORM;
  b = orc_mas_field(mas, 2, rr, th, ph);
  out->br = b * sqrt(4.0 * ORC_PI * ORC_MAS_RHO_NORM) * ORC_MAS_LENGTH_NORM / ORC_MAS_TIME_NORM / ORC_MHD_B_NORM;
  b = orc_mas_field(mas, 3, rr, th, ph);
  out->vp = b * (ORC_MAS_LENGTH_NORM / ORC_MAS_TIME_NORM) / ORC_C;
  b = orc_mas_field(mas, 4, rr, th, ph);
  out->vt = b * (ORC_MAS_LENGTH_NORM / ORC_MAS_TIME_NORM) / ORC_C;
  b = orc_mas_field(mas, 5, rr, th, ph);
  out->vr = b * (ORC_MAS_LENGTH_NORM / ORC_MAS_TIME_NORM) / ORC_C;
  if (out->vr < (mas->p.v_min / ORC_C)) out->vr = (mas->p.v_min / ORC_C);
  b = orc_mas_field(mas, 6, rr, th, ph);
  out->d = b * (ORC_MAS_RHO_NORM / ORC_MP) / ORC_MHD_DENSITY_NORM;
}

/* masWind, src/masInterp.c:1007-1065: Parker extrapolation from the node's
 * previous values. */
static void orc_mas_wind(const orc_mas_t *mas, const eprem_params_t *p, const double *nodes,
                         size_t SN, size_t g, orc_masnode_t *out) {
  const double *F = nodes;
#define NF(field) F[(size_t)(field) * SN + g]
  double ox = NF(EPREM_NODE_ROLD_X), oy = NF(EPREM_NODE_ROLD_Y), oz = NF(EPREM_NODE_ROLD_Z);
  double br = NF(EPREM_NODE_BR), bt = NF(EPREM_NODE_BTHETA), bp = NF(EPREM_NODE_BPHI);
  double vr = NF(EPREM_NODE_VR), vt = NF(EPREM_NODE_VTHETA), vp = NF(EPREM_NODE_VPHI);
  double rho = NF(EPREM_NODE_DENSITY);
  double rOldmag = sqrt(ox * ox + oy * oy + oz * oz);
  double rmag = NF(EPREM_NODE_RMAG);
  double oneOverR = rOldmag / rmag;
  out->br = br * oneOverR * oneOverR;
  out->bt = bt * oneOverR;
  out->bp = bp * oneOverR;
  if ((mas->p.cor_rotate_fake > 0) && (mas->p.rotate_solution > 0)) {
    double theta = acos(NF(EPREM_NODE_RZ) / rmag);
    double thetaOld = acos(oz / rOldmag);
    out->bp += ((p->r_scale * p->omega_sun / vr) *
                (rOldmag * br * sin(thetaOld) - rmag * out->br * sin(theta)));
  }
  out->vr = vr;
  out->vt = vt * oneOverR;
  out->vp = vp * oneOverR;
  out->d = rho * oneOverR * oneOverR;
#undef NF
}

/* cartToSphPosAu, src/geometry.c:131-157 */
static void orc_sph_au(const eprem_params_t *p, double x, double y, double z, double *r,
                       double *th, double *ph) {
  double ax = x * p->r_scale, ay = y * p->r_scale, az = z * p->r_scale;
  *r = sqrt(ax * ax + ay * ay + az * az);
  *th = acos(az / *r);
  *ph = atan2(ay, ax);
  while (*ph < 0.0) *ph += (2.0 * ORC_PI);
  if (*ph < 0.0)
    while (*ph < 0.0) *ph += 2 * ORC_PI;
  if (*ph > 2 * ORC_PI)
    while (*ph > 2 * ORC_PI) *ph -= 2 * ORC_PI;
}

/* masGetNode, src/masInterp.c:31-68 (no heliospheric domain). */
static void orc_mas_get_node(const orc_mas_t *mas, const eprem_params_t *p, const double *nodes,
                             size_t SN, size_t g, double pr, double pth, double pph,
                             orc_masnode_t *out) {
  if (pr <= (mas->p.radial_max * ORC_RSAU))
    orc_mas_trilinear(mas, pr, pth, pph, out);
  else
    orc_mas_wind(mas, p, nodes, SN, g, out);
}

int orc_mas_update_mhd(const eprem_dims_t *d, const eprem_params_t *p, double *nodes,
                       const orc_mas_t *mas, double t_global) {
  (void)t_global;
  const int N = d->num_nodes;
  const size_t SN = (size_t)d->num_streams * N;
  for (int s = 0; s < d->num_streams; s++)
    for (int k = 0; k < N; k++) {
      const size_t g = (size_t)s * N + k;
      NODE(EPREM_NODE_BMAG_OLD, s, k) = NODE(EPREM_NODE_BMAG, s, k);
      NODE(EPREM_NODE_DENSITY_OLD, s, k) = NODE(EPREM_NODE_DENSITY, s, k);
      NODE(EPREM_NODE_VSPH_OLD_R, s, k) = NODE(EPREM_NODE_VR, s, k);
      NODE(EPREM_NODE_VSPH_OLD_THETA, s, k) = NODE(EPREM_NODE_VTHETA, s, k);
      NODE(EPREM_NODE_VSPH_OLD_PHI, s, k) = NODE(EPREM_NODE_VPHI, s, k);
      NODE(EPREM_NODE_DS_OLD, s, k) = NODE(EPREM_NODE_DS, s, k);
      NODE(EPREM_NODE_ROLDER_X, s, k) = NODE(EPREM_NODE_RX, s, k);
      NODE(EPREM_NODE_ROLDER_Y, s, k) = NODE(EPREM_NODE_RY, s, k);
      NODE(EPREM_NODE_ROLDER_Z, s, k) = NODE(EPREM_NODE_RZ, s, k);
      double x = NODE(EPREM_NODE_RX, s, k), y = NODE(EPREM_NODE_RY, s, k),
             z = NODE(EPREM_NODE_RZ, s, k), rmag = NODE(EPREM_NODE_RMAG, s, k);
      double pr, pth, pph;
      orc_sph_au(p, x, y, z, &pr, &pth, &pph);
      orc_masnode_t mn;
      orc_mas_get_node(mas, p, nodes, SN, g, pr, pth, pph, &mn);
      double dens = mn.d;
      NODE(EPREM_NODE_DENSITY, s, k) = dens;
      if (dens <= 0.0)
        NODE(EPREM_NODE_DIVV, s, k) = 0.0;
      else
        NODE(EPREM_NODE_DIVV, s, k) = -1.0 * log(dens / NODE(EPREM_NODE_DENSITY_OLD, s, k)) / p->t_del;
      double theta = acos(z / rmag);
      double phi = atan2(y, x);
      double Vr = mn.vr, Vt = mn.vt, Vp = mn.vp;
      NODE(EPREM_NODE_VR, s, k) = Vr;
      NODE(EPREM_NODE_VTHETA, s, k) = Vt;
      NODE(EPREM_NODE_VPHI, s, k) = Vp;
      NODE(EPREM_NODE_VMAG, s, k) = sqrt(Vr * Vr + Vt * Vt + Vp * Vp);
      NODE(EPREM_NODE_VVEC_X, s, k) = Vr * sin(theta) * cos(phi) + Vt * cos(theta) * cos(phi) - Vp * sin(phi);
      NODE(EPREM_NODE_VVEC_Y, s, k) = Vr * sin(theta) * sin(phi) + Vt * cos(theta) * sin(phi) + Vp * cos(phi);
      NODE(EPREM_NODE_VVEC_Z, s, k) = Vr * cos(theta) - Vt * sin(theta);
      double Br = mn.br, Bt = mn.bt, Bp = mn.bp;
      NODE(EPREM_NODE_BR, s, k) = Br;
      NODE(EPREM_NODE_BTHETA, s, k) = Bt;
      NODE(EPREM_NODE_BPHI, s, k) = Bp;
      double Bmag = sqrt(Br * Br + Bt * Bt + Bp * Bp);
      NODE(EPREM_NODE_BMAG, s, k) = Bmag;
      NODE(EPREM_NODE_BVEC_X, s, k) = Br * sin(theta) * cos(phi) + Bt * cos(theta) * cos(phi) - Bp * sin(phi);
      NODE(EPREM_NODE_BVEC_Y, s, k) = Br * sin(theta) * sin(phi) + Bt * cos(theta) * sin(phi) + Bp * cos(phi);
      NODE(EPREM_NODE_BVEC_Z, s, k) = Br * cos(theta) - Bt * sin(theta);
      if (k == 0) {
        NODE(EPREM_NODE_DUPAR, s, k) = 0.0;
        NODE(EPREM_NODE_DLNB, s, k) = 0.0;
        NODE(EPREM_NODE_DLNN, s, k) = 0.0;
      } else {
        double dupar = (Vr - NODE(EPREM_NODE_VSPH_OLD_R, s, k)) * Br +
                       (Vt - NODE(EPREM_NODE_VSPH_OLD_THETA, s, k)) * Bt +
                       (Vp - NODE(EPREM_NODE_VSPH_OLD_PHI, s, k)) * Bp;
        dupar /= Bmag;
        NODE(EPREM_NODE_DUPAR, s, k) = dupar;
        NODE(EPREM_NODE_DLNB, s, k) = log(Bmag / NODE(EPREM_NODE_BMAG_OLD, s, k));
        NODE(EPREM_NODE_DLNN, s, k) = log(dens / NODE(EPREM_NODE_DENSITY_OLD, s, k));
      }
    }
  return EPREM_GPU_OK;
}

/* sphToCartVector, src/geometry.c:89-121 */
static void orc_sph_to_cart_vec(double vr, double vt, double vp, double x, double y, double z,
                                double *ox, double *oy, double *oz) {
  double rmag = sqrt(x * x + y * y + z * z);
  if ((rmag - fabs(z)) < ORC_VERYSMALL) {
    *ox = 0.0;
    *oy = 0.0;
  } else {
    *ox = x / rmag * vr + x * z / (rmag * sqrt(rmag * rmag - z * z)) * vt -
          y / sqrt(rmag * rmag - z * z) * vp;
    *oy = y / rmag * vr + y * z / (rmag * sqrt(rmag * rmag - z * z)) * vt +
          x / sqrt(rmag * rmag - z * z) * vp;
  }
  *oz = z / rmag * vr - sqrt(rmag * rmag - z * z) / rmag * vt;
}

/* vMas, src/masInterp.c:1281-1296: velocity at position (x,y,z) for node g
 * (whose stored fields feed masWind beyond the MAS domain). */
static void orc_vmas(const orc_mas_t *mas, const eprem_params_t *p, const double *nodes,
                     size_t SN, size_t g, double x, double y, double z, double *vx, double *vy,
                     double *vz) {
  double pr, pth, pph;
  orc_sph_au(p, x, y, z, &pr, &pth, &pph);
  orc_masnode_t mn;
  orc_mas_get_node(mas, p, nodes, SN, g, pr, pth, pph, &mn);
  orc_sph_to_cart_vec(mn.vr, mn.vt, mn.vp, x, y, z, vx, vy, vz);
}

int orc_mas_move_nodes(const eprem_dims_t *d, const eprem_params_t *p, double *nodes,
                       const orc_mas_t *mas, double dt) {
  const int N = d->num_nodes;
  const size_t SN = (size_t)d->num_streams * N;
  const double sixth = 1.0 / 6.0, two = 2.0, half = 0.5;
  for (int s = 0; s < d->num_streams; s++)
    for (int k = 1; k < N; k++) {
      const size_t g = (size_t)s * N + k;
      double x0 = NODE(EPREM_NODE_RX, s, k), y0 = NODE(EPREM_NODE_RY, s, k),
             z0 = NODE(EPREM_NODE_RZ, s, k);
      /* rungeKuttaFlow (src/masInterp.c:1306-1334) reads the node as it was
       * before this call set rOld, so rOld is written after the push. */
      double vx, vy, vz, k1x, k1y, k1z, k2x, k2y, k2z, k3x, k3y, k3z, k4x, k4y, k4z;
      orc_vmas(mas, p, nodes, SN, g, x0, y0, z0, &vx, &vy, &vz);
      k1x = vx * (dt / p->r_scale); k1y = vy * (dt / p->r_scale); k1z = vz * (dt / p->r_scale);
      orc_vmas(mas, p, nodes, SN, g, x0 + k1x * half, y0 + k1y * half, z0 + k1z * half, &vx, &vy, &vz);
      k2x = vx * (dt / p->r_scale); k2y = vy * (dt / p->r_scale); k2z = vz * (dt / p->r_scale);
      orc_vmas(mas, p, nodes, SN, g, x0 + k2x * half, y0 + k2y * half, z0 + k2z * half, &vx, &vy, &vz);
      k3x = vx * (dt / p->r_scale); k3y = vy * (dt / p->r_scale); k3z = vz * (dt / p->r_scale);
      orc_vmas(mas, p, nodes, SN, g, x0 + k3x, y0 + k3y, z0 + k3z, &vx, &vy, &vz);
      k4x = vx * (dt / p->r_scale); k4y = vy * (dt / p->r_scale); k4z = vz * (dt / p->r_scale);
      double x1 = x0 + sixth * (k1x + two * k2x + two * k3x + k4x);
      double y1 = y0 + sixth * (k1y + two * k2y + two * k3y + k4y);
      double z1 = z0 + sixth * (k1z + two * k2z + two * k3z + k4z);
      NODE(EPREM_NODE_ROLD_X, s, k) = x0;
      NODE(EPREM_NODE_ROLD_Y, s, k) = y0;
      NODE(EPREM_NODE_ROLD_Z, s, k) = z0;
      NODE(EPREM_NODE_RX, s, k) = x1;
      NODE(EPREM_NODE_RY, s, k) = y1;
      NODE(EPREM_NODE_RZ, s, k) = z1;
      NODE(EPREM_NODE_RMAG, s, k) = sqrt((x1 * x1) + (y1 * y1) + (z1 * z1));
    }
  return EPREM_GPU_OK;
}
