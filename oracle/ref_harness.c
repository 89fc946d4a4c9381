/*
 * ref_harness.c -- drives the EPREM reference's own hot-path functions,
 * compiled from the reference source tree by oracle/Makefile into
 * oracle/_ref/libeprem_ref.so.  TEST INFRASTRUCTURE ONLY: it exists to pin
 * the CPU restatement (eprem_oracle.c) against the reference itself.
 *
 * With ref_shims.c (one-rank MPI, config reader, netCDF capture) it
 * supplies what the reference links against but the container lacks, plus
 * the timer globals that src/eprem.c defines; the harness fills the
 * reference's `config` struct directly and asks for no file I/O.
 * and a small C API (ref_*) that loads a state in the include/eprem_gpu.h
 * layout into the reference globals, calls the reference entry points
 * (updateEnergeticParticles, updateMhd, moveNodes) and reads the state back.
 */
#include <float.h>
#include <math.h>
#include <setjmp.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "mpi.h"
#include "libconfig.h"
#include "netcdf.h"
#include "hdf5.h"

#include "baseTypes.h"
#include "configuration.h"
#include "cubeShellInit.h"
#include "cubeShellStruct.h"
#include "energeticParticles.h"
#include "energeticParticlesInit.h"
#include "energeticParticlesTypes.h"
#include "flow.h"
#include "global.h"
#include "mpiInit.h"
#include "simCore.h"
#include "unifiedOutput.h"
#include "readMAS.h"
#include "masInterp.h"

#include "../include/eprem_gpu.h"

/* ---- timers (defined by src/eprem.c:409-423 in the reference binary) ---- */
double timer_diffusestream, timer_adiabaticfocus, timer_adiabaticchange,
    timer_diffuseshell, timer_driftshell, timer_eptotal, timer_mas_io,
    timer_eprem_io, timer_init, timer_other, timer_wall, timer_start,
    timer_MPIgatherscatter, timer_MPIsendrecv;

extern Index_t maxsubcycles_energychange, maxsubcycles_focusing;
extern Scalar_t min_tau;
extern Index_t **computeLines;

/* ---- abort trap: panic() ends in MPI_Abort ------------------------------ */
static jmp_buf ref_abort_jmp;
static int ref_abort_armed = 0;

/* MPI, libconfig, netCDF and HDF5 come from ref_shims.c. */
extern void (*refshim_abort_hook)(int code);
extern size_t refshim_type_size(MPI_Datatype t);
static void ref_abort(int code) {
  if (ref_abort_armed) longjmp(ref_abort_jmp, code);
}

/* ---- harness API -------------------------------------------------------- */
static int ref_S = 0, ref_N = 0;
static double ref_mass[1], ref_charge[1];

/* Configure the reference globals as getParams + setRuntimeConstants
 * (src/configuration.c:43-348) would for a one-rank run, then run the
 * reference's own initialisation: initMPIOffsets, allocateGlobalVariables,
 * initMPITypes, flagParamInit, defineComputeLines, simCoreInit,
 * initEnergeticParticlesGrids (src/eprem.c:440-475). */
int ref_setup(int rows, int cols, const eprem_dims_t *d, const eprem_params_t *p,
              double e_min, double e_max, double mass, double charge, double rigidity_power) {
  static int done = 0;
  if (done) return -100; /* the reference allocates its globals once per process */
  done = 1;
  memset(&config, 0, sizeof(config));
  config.numNodesPerStream = d->num_nodes;
  config.numRowsPerFace = rows;
  config.numColumnsPerFace = cols;
  config.numEnergySteps = d->num_energies;
  config.numMuSteps = d->num_mu;
  config.adiabaticChangeAlg = p->adiabatic_change_alg;
  config.adiabaticFocusAlg = p->adiabatic_focus_alg;
  config.rScale = p->r_scale;
  config.tDel = p->t_del;
  config.numEpSteps = p->num_ep_steps;
  config.omegaSun = p->omega_sun;
  config.lamo = p->lamo;
  config.dsh_min = p->dsh_min;
  config.dsh_hel_min = 2.5e-4;
  config.mfpType = p->mfp_type;
  config.mfpRadialPower = p->mfp_radial_power;
  config.mfpBPower = p->mfp_b_power;
  config.rigidityPower = rigidity_power;
  config.eMin = e_min;
  config.eMax = e_max;
  config.useEPBoundary = p->use_ep_boundary;
  config.checkSeedPopulation = p->check_seed_population;
  config.useAdiabaticChange = p->use_adiabatic_change;
  config.dampCooling = p->damp_cooling;
  config.useAdiabaticFocus = p->use_adiabatic_focus;
  config.useShellDiffusion = 0;
  config.useParallelDiffusion = p->use_parallel_diffusion;
  config.useDrift = 0;
  config.numSpecies = 1;
  ref_mass[0] = mass;
  ref_charge[0] = charge;
  config.mass = ref_mass;
  config.charge = ref_charge;
  config.masCouple = 0;
  config.masHelCouple = 0;
  config.useBoundaryFunction = p->use_boundary_function;
  config.boundaryFunctionInitDomain = 1;
  config.boundaryFunctAmplitude = p->bf_amplitude;
  config.boundaryFunctXi = p->bf_xi;
  config.boundaryFunctGamma = p->bf_gamma;
  config.boundaryFunctBeta = p->bf_beta;
  config.boundaryFunctEcutoff = p->bf_ecutoff;
  config.boundaryFunctR0 = p->bf_r0;
  config.idealShock = p->ideal_shock;
  config.idealShockSharpness = p->ideal_shock_sharpness;
  config.idealShockScaleLength = p->ideal_shock_scale_length;
  config.idealShockJump = p->ideal_shock_jump;
  config.idealShockFalloff = p->ideal_shock_falloff;
  config.idealShockSpeed = p->ideal_shock_speed;
  config.idealShockInitTime = p->ideal_shock_init_time;
  config.idealShockTheta = p->ideal_shock_theta;
  config.idealShockPhi = p->ideal_shock_phi;
  config.idealShockWidth = p->ideal_shock_width;
  config.mhdUs = p->mhd_us;
  config.mhdNsAu = p->mhd_ns_au;
  config.mhdBsAu = p->mhd_bs_au;
  /* setRuntimeConstants, src/configuration.c:328-337 */
  FACE_ROWS = rows;
  FACE_COLS = cols;
  NUM_SPECIES = 1;
  NUM_ESTEPS = d->num_energies;
  NUM_MUSTEPS = d->num_mu;
  NUM_OBS = 0;
  AdiabaticChangeAlg = p->adiabatic_change_alg;
  AdiabaticFocusAlg = p->adiabatic_focus_alg;
  TOTAL_NUM_SHELLS = d->num_nodes;
  /* initMPI, src/mpiInit.c:50-67, one rank */
  mpi_rank = 0;
  N_PROCS = 1;
  initMPIOffsets();
  allocateGlobalVariables();
  initMPITypes();
  flagParamInit();
  defineComputeLines();
  simCoreInit();
  initEnergeticParticlesGrids();
  ref_S = NUM_STREAMS;
  ref_N = d->num_nodes;
  if (ref_S != d->num_streams) return -101;
  if (LOCAL_NUM_SHELLS != ref_N + 1) return -102;
  return 0;
}

int ref_get_grids(double *eg, double *vg, double *vgi, double *mug, double *rig, double *out_dlnp,
                  double *out_dmu) {
  for (int e = 0; e < NUM_ESTEPS; e++) {
    eg[e] = egrid[e];
    vg[e] = vgrid[e];
    vgi[e] = vgrid_i[e];
    rig[e] = rigidity[e];
  }
  for (int m = 0; m < NUM_MUSTEPS; m++) mug[m] = mugrid[m];
  *out_dlnp = dlnp;
  *out_dmu = dmu;
  return 0;
}

/* Node_t member for each eprem_node_field. */
static double *node_member(Node_t *n, int field) {
  switch (field) {
    case EPREM_NODE_RX: return &n->r.x;
    case EPREM_NODE_RY: return &n->r.y;
    case EPREM_NODE_RZ: return &n->r.z;
    case EPREM_NODE_RMAG: return &n->rmag;
    case EPREM_NODE_BMAG: return &n->mhdBmag;
    case EPREM_NODE_DLNB: return &n->mhdDlnB;
    case EPREM_NODE_DLNN: return &n->mhdDlnN;
    case EPREM_NODE_DUPAR: return &n->mhdDuPar;
    case EPREM_NODE_DS: return &n->ds;
    case EPREM_NODE_BMAG_PLUS: return &n->mhdBmagPlus;
    case EPREM_NODE_BMAG_MINUS: return &n->mhdBmagMinus;
    case EPREM_NODE_BR: return &n->mhdBr;
    case EPREM_NODE_BTHETA: return &n->mhdBtheta;
    case EPREM_NODE_BPHI: return &n->mhdBphi;
    case EPREM_NODE_VR: return &n->mhdVr;
    case EPREM_NODE_VTHETA: return &n->mhdVtheta;
    case EPREM_NODE_VPHI: return &n->mhdVphi;
    case EPREM_NODE_VMAG: return &n->mhdVmag;
    case EPREM_NODE_DENSITY: return &n->mhdDensity;
    case EPREM_NODE_DIVV: return &n->mhdDivV;
    case EPREM_NODE_BVEC_X: return &n->mhdBvec.x;
    case EPREM_NODE_BVEC_Y: return &n->mhdBvec.y;
    case EPREM_NODE_BVEC_Z: return &n->mhdBvec.z;
    case EPREM_NODE_VVEC_X: return &n->mhdVvec.x;
    case EPREM_NODE_VVEC_Y: return &n->mhdVvec.y;
    case EPREM_NODE_VVEC_Z: return &n->mhdVvec.z;
    case EPREM_NODE_BMAG_OLD: return &n->mhdBmagOld;
    case EPREM_NODE_DENSITY_OLD: return &n->mhdDensityOld;
    case EPREM_NODE_VSPH_OLD_R: return &n->mhdVsphOld.r;
    case EPREM_NODE_VSPH_OLD_THETA: return &n->mhdVsphOld.theta;
    case EPREM_NODE_VSPH_OLD_PHI: return &n->mhdVsphOld.phi;
    case EPREM_NODE_DS_OLD: return &n->dsOld;
    case EPREM_NODE_ROLD_X: return &n->rOld.x;
    case EPREM_NODE_ROLD_Y: return &n->rOld.y;
    case EPREM_NODE_ROLD_Z: return &n->rOld.z;
    case EPREM_NODE_ROLDER_X: return &n->rOlder.x;
    case EPREM_NODE_ROLDER_Y: return &n->rOlder.y;
    case EPREM_NODE_ROLDER_Z: return &n->rOlder.z;
  }
  return NULL;
}

/* Node k of stream s is grid shell k+1 (shell 0 is the spawn template,
 * INNER_SHELL, which the hot path never reads). */
int ref_load(const double *f, const double *nodes) {
  const size_t SN = (size_t)ref_S * ref_N;
  const int EM = NUM_ESTEPS * NUM_MUSTEPS;
  for (int s = 0; s < ref_S; s++) {
    Node_t *g0 = &grid[(size_t)s * LOCAL_NUM_SHELLS];
    memset(g0, 0, sizeof(Node_t));
    for (int i = 0; i < EM; i++) eParts[(size_t)s * SSPEM + i] = DBL_MIN;
    for (int k = 0; k < ref_N; k++) {
      Node_t *n = &grid[(size_t)s * LOCAL_NUM_SHELLS + k + 1];
      for (int fld = 0; fld < EPREM_NODE_NFIELDS; fld++)
        *node_member(n, fld) = nodes[(size_t)fld * SN + (size_t)s * ref_N + k];
      memcpy(&eParts[(size_t)s * SSPEM + (size_t)(k + 1) * EM], &f[((size_t)s * ref_N + k) * EM],
             sizeof(double) * EM);
    }
  }
  return 0;
}

int ref_store(double *f, double *nodes) {
  const size_t SN = (size_t)ref_S * ref_N;
  const int EM = NUM_ESTEPS * NUM_MUSTEPS;
  for (int s = 0; s < ref_S; s++)
    for (int k = 0; k < ref_N; k++) {
      Node_t *n = &grid[(size_t)s * LOCAL_NUM_SHELLS + k + 1];
      for (int fld = 0; fld < EPREM_NODE_NFIELDS; fld++)
        nodes[(size_t)fld * SN + (size_t)s * ref_N + k] = *node_member(n, fld);
      memcpy(&f[((size_t)s * ref_N + k) * EM], &eParts[(size_t)s * SSPEM + (size_t)(k + 1) * EM],
             sizeof(double) * EM);
    }
  return 0;
}

/* Switch useShellDiffusion on (on = 1) with config.kperxkpar: the grid gets
 * the reference's own NEWS links (initNEWS on the inner shell, then
 * initCopyAll to every shell, as gridStructInit does, src/cubeShellInit.c:
 * 46-94), returned in news as stream indices face*R*C + row*C + col, four per
 * stream in the order north, east, west, south.  initCopyAll also places the
 * nodes on the unit sphere; ref_load sets them afterwards. */
static int ref_news_ready = 0;
static void ref_news(int32_t *news) {
  if (!ref_news_ready) {
    initNEWS(INNER_SHELL);
    initCopyAll();
    ref_news_ready = 1;
  }
  for (int s = 0; s < ref_S; s++) {
    const Node_t *n = &grid[(size_t)s * LOCAL_NUM_SHELLS + INNER_ACTIVE_SHELL];
    const Neighbor_t *nb[4] = {&n->n, &n->e, &n->w, &n->s};
    for (int d = 0; d < 4; d++)
      news[s * 4 + d] = (int32_t)((nb[d]->face * FACE_ROWS + nb[d]->row) * FACE_COLS + nb[d]->col);
  }
}

/* useDrift on or off, with the grid's NEWS links (news) and the momentum
 * grid's lnpmin (the reference's global) handed back. */
int ref_drift(int on, int32_t *news, double *lnpmin_out) {
  ref_news(news);
  config.useDrift = on;
  *lnpmin_out = lnpmin;
  return 0;
}

int ref_shell_diffusion(int on, double kperxkpar, int32_t *news) {
  ref_news(news);
  config.useShellDiffusion = on;
  config.kperxkpar = kperxkpar;
  return 0;
}

/* The reference entry points.  A panic inside returns its MPI_Abort code.
 * With useShellDiffusion on, ShellData runs first, as the driver calls it
 * right before updateEnergeticParticles (src/eprem.c:647-671). */
int ref_update_energetic_particles(double tg, eprem_ep_stats_t *st) {
  t_global = tg;
  maxsubcycles_energychange = 0;
  maxsubcycles_focusing = 0;
  min_tau = DBL_MAX;
  refshim_abort_hook = ref_abort;
  ref_abort_armed = 1;
  int code = setjmp(ref_abort_jmp);
  if (code == 0) {
    if (config.useShellDiffusion > 0 || config.useDrift > 0) ShellData();
    updateEnergeticParticles();
  }
  ref_abort_armed = 0;
  st->max_subcycles_change = maxsubcycles_energychange;
  st->max_subcycles_focusing = maxsubcycles_focusing;
  st->min_tau = min_tau;
  return code;
}

int ref_update_mhd(double tg) {
  t_global = tg;
  updateMhd();
  return 0;
}

int ref_move_nodes(double dt) {
  moveNodes(dt);
  return 0;
}

int ref_node_t_size(void) { return (int)sizeof(Node_t); }
int ref_node_T_extent(void) { return (int)refshim_type_size(Node_T); }

/* ---- MAS background ------------------------------------------------------ */
/* Point the reference's MAS globals (src/readMAS.h) at caller arrays, as
 * masGetInterpData leaves them after reading two slices, and switch updateMhd
 * to its MHD_MAS branch. */
int ref_mas_setup(const eprem_mas_params_t *mp, const eprem_mas_slice_t *a,
                  const eprem_mas_slice_t *b, double scor, double phioff) {
  config.masCouple = 1;
  config.masHelCouple = 0;
  config.masRadialMax = mp->radial_max;
  config.masVmin = mp->v_min;
  config.masCorRotateFake = mp->cor_rotate_fake;
  config.masRotateSolution = mp->rotate_solution;
  mhdGridStatus = MHD_MAS;
  s_cor = scor;
  phiOffset = phioff;
#define SETF(F, i, S, sl)                                      \
  mas##F##_##sl = (float *)S->data[i];                         \
  mas##F##rDim_##sl = (float *)S->mesh[i][0];                  \
  mas##F##tDim_##sl = (float *)S->mesh[i][1];                  \
  mas##F##pDim_##sl = (float *)S->mesh[i][2];                  \
  mas##F##rDimMax_##sl[0] = S->dims[i][0];                     \
  mas##F##tDimMax_##sl[0] = S->dims[i][1];                     \
  mas##F##pDimMax_##sl[0] = S->dims[i][2];
  SETF(Bp, 0, a, 0) SETF(Bt, 1, a, 0) SETF(Br, 2, a, 0) SETF(Vp, 3, a, 0) SETF(Vt, 4, a, 0)
  SETF(Vr, 5, a, 0) SETF(D, 6, a, 0)
  SETF(Bp, 0, b, 1) SETF(Bt, 1, b, 1) SETF(Br, 2, b, 1) SETF(Vp, 3, b, 1) SETF(Vt, 4, b, 1)
  SETF(Vr, 5, b, 1) SETF(D, 6, b, 1)
#undef SETF
  masDimMin_0[0] = 0;
  masDimMin_1[0] = 0;
  return 0;
}

int ref_mas_move_nodes(double dt) {
  masMoveNodes(dt);
  return 0;
}
