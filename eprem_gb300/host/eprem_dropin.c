/*
 * eprem_dropin.c -- the GB300 path behind EPREM's own hot-path entry points.
 *
 * Link this file and libeprem_gpu.so into the reference build in place of the
 * bodies of
 *   updateEnergeticParticles()  src/energeticParticles.c:70-203
 *   updateMhd()                 src/flow.c:36-154
 *   moveNodes(dt)               src/simCore.c:737-785
 *   masMoveNodes(dt)            src/masInterp.c:1344-1393
 *   rotSunAndSpawnShell(dt)     src/simCore.c:443-630
 * and around
 *   dataDumpIO()                src/unifiedOutput.c:1479-1531
 *   initEnergeticParticles()    src/energeticParticlesInit.c:103-147
 * (the originals are renamed with -D at compile time so that the driver
 * src/eprem.c, unchanged, calls these).
 *
 * f lives on the device from the first shell ripple on: the EP update works
 * on it there, rotSunAndSpawnShell ripples it there (the grid still ripples
 * on the host), and eParts is brought up to date only before the driver
 * reads it, in dataDumpIO.  The driver writes eParts only through
 * initEnergeticParticles (after seeding, at the first EP step, and after
 * every step of the seed test); the device copy is dropped then and taken
 * again at its next use.
 *
 * The reference keeps its state in globals (grid[], eParts[], config, the
 * 1-D grids of energeticParticlesTypes.h); each call here packs what the GPU
 * needs into the plain arrays of include/eprem_gpu.h, runs the GPU entry
 * point and unpacks the results, so everything else in the driver -- output,
 * shell spawning, MAS reading -- sees the same globals as before.
 *
 * MAS runs: masGetInterpData (src/readMAS.c:645-998) still reads the slice
 * files into the reference's _0 / _1 globals; a slot is copied to the device
 * when its file index (masFileIndex0 / masFileIndex1) changes, and s_cor and
 * phiOffset are passed on every call.
 *
 * Output: dataDumpIO brings f down only when an output is due, and with
 * streamFluxOutput alone only the device's omnidirectional flux (1/M of f).
 *
 * Scope: one MPI rank holds every stream (the GPU replaces the rank
 * decomposition), one species, analytic or MAS coronal background (the
 * heliospheric MAS coupling is refused with the reference's panic), shell
 * diffusion and drift (drift with the analytic background only).
 */
#include <float.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "baseTypes.h"
#include "configuration.h"
#include "cubeShellStruct.h"
#include "energeticParticles.h"
#include "energeticParticlesTypes.h"
#include "error.h"
#include "flow.h"
#include "global.h"
#include "masInterp.h"
#include "mpiInit.h"
#include "readMAS.h"
#include "simCore.h"
#include "timers.h"

#include "eprem_gpu.h"

/* The reference's own output routine and seed-population initialisation,
 * renamed at compile time (-DdataDumpIO=dataDumpIO_cpu on
 * src/unifiedOutput.c, -DinitEnergeticParticles=initEnergeticParticles_cpu on
 * src/energeticParticlesInit.c). */
void dataDumpIO_cpu(void);
void initEnergeticParticles_cpu(void);

static eprem_gpu_run *dropin_run = NULL;
static double dropin_t_del = 0.0;   /* config.tDel as last passed to the run */
static int dropin_f_dev = 0;        /* the device holds f (eParts shells 1..N) */
static int dropin_f_stale = 0;      /* eParts is older than the device's f     */
static double *dropin_nodes = NULL; /* [field][S*N] host staging of grid[]   */
static size_t dropin_sn = 0;

static void dropin_check(int rc, const char *what) {
  if (rc != EPREM_GPU_OK) {
    static char msg[512];
    snprintf(msg, sizeof(msg), "%s: %s", what, eprem_gpu_last_error());
    panic(msg);
  }
}

/* Node_t member for each eprem_node_field (src/cubeShellStruct.h:51-93). */
static double *dropin_member(Node_t *n, int field) {
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

/* First call: size the run from the reference globals and create it. */
static void dropin_init(void) {
  if (dropin_run) return;
  if (N_PROCS != 1) panic("GPU path: run with one MPI rank (every stream lives on the GPU)");
  if (config.masHelCouple > 0)
    panic("GPU path: heliospheric MAS coupling is not supported by this build");

  eprem_dims_t d;
  d.num_streams = NUM_STREAMS;
  d.num_nodes = TOTAL_NUM_SHELLS;
  d.num_species = NUM_SPECIES;
  d.num_energies = NUM_ESTEPS;
  d.num_mu = NUM_MUSTEPS;
  d.precision = getenv("EPREM_GPU_FP32") ? EPREM_FP32 : EPREM_FP64;
  eprem_params_t p;
  memset(&p, 0, sizeof(p));
  p.r_scale = config.rScale;
  p.t_del = config.tDel;
  p.num_ep_steps = config.numEpSteps;
  p.use_parallel_diffusion = config.useParallelDiffusion;
  p.use_adiabatic_focus = config.useAdiabaticFocus;
  p.use_adiabatic_change = config.useAdiabaticChange;
  p.check_seed_population = config.checkSeedPopulation;
  p.use_ep_boundary = config.useEPBoundary;
  p.use_boundary_function = config.useBoundaryFunction;
  p.adiabatic_focus_alg = config.adiabaticFocusAlg;
  p.adiabatic_change_alg = config.adiabaticChangeAlg;
  p.damp_cooling = config.dampCooling;
  p.dsh_min = config.dsh_min;
  p.mfp_type = config.mfpType;
  p.lamo = config.lamo;
  p.mfp_radial_power = config.mfpRadialPower;
  p.mfp_b_power = config.mfpBPower;
  p.mhd_bs_au = config.mhdBsAu;
  p.bf_amplitude = config.boundaryFunctAmplitude;
  p.bf_xi = config.boundaryFunctXi;
  p.bf_gamma = config.boundaryFunctGamma;
  p.bf_beta = config.boundaryFunctBeta;
  p.bf_ecutoff = config.boundaryFunctEcutoff;
  p.bf_r0 = config.boundaryFunctR0;
  p.mhd_us = config.mhdUs;
  p.mhd_ns_au = config.mhdNsAu;
  p.omega_sun = config.omegaSun;
  p.ideal_shock = config.idealShock;
  p.ideal_shock_sharpness = config.idealShockSharpness;
  p.ideal_shock_scale_length = config.idealShockScaleLength;
  p.ideal_shock_jump = config.idealShockJump;
  p.ideal_shock_falloff = config.idealShockFalloff;
  p.ideal_shock_speed = config.idealShockSpeed;
  p.ideal_shock_init_time = config.idealShockInitTime;
  p.ideal_shock_theta = config.idealShockTheta;
  p.ideal_shock_phi = config.idealShockPhi;
  p.ideal_shock_width = config.idealShockWidth;
  p.max_subcycles = 0;
  eprem_grids_t g;
  g.egrid = egrid;
  g.vgrid = vgrid;
  g.vgrid_i = vgrid_i;
  g.mugrid = mugrid;
  g.rigidity = rigidity;
  g.dlnp = dlnp;
  g.dmu = dmu;
  dropin_check(eprem_gpu_create(&d, &p, &g, &dropin_run), "eprem_gpu_create");
  /* useDrift: curl(B)/B^2 from every updateMhd from here on; the drift
   * itself once the grid's links exist (dropin_perp_setup) */
  if (config.useDrift > 0) {
    eprem_drift_params_t dp;
    dp.lnpmin = lnpmin;
    dp.charge = config.charge[0];
    dp.mass = config.mass[0];
    dropin_check(eprem_gpu_set_drift(dropin_run, NULL, &dp), "drift");
  }
  dropin_t_del = config.tDel;
  dropin_sn = (size_t)d.num_streams * d.num_nodes;
  dropin_nodes = (double *)eprem_gpu_host_alloc(sizeof(double) * EPREM_NODE_NFIELDS * dropin_sn);
  if (!dropin_nodes) panic("GPU path: host staging allocation failed");
  /* f moves straight between eParts and the device (no host staging); lock
   * eParts in place so those copies overlap the update -- if it cannot be
   * locked they stay correct, only slower */
  if (eprem_gpu_host_register(eParts, sizeof(Scalar_t) * (size_t)NUM_STREAMS * SSPEM) !=
      EPREM_GPU_OK)
    fprintf(stderr, "GPU path: eParts not page-locked (%s); copies will not overlap\n",
            eprem_gpu_last_error());
}

/* SetDT (src/simCore.c:800-880) changes config.tDel between steps of a
 * MAS-coupled run: pass the current value on before each call. */
static void dropin_sync_step(void) {
  if (config.tDel != dropin_t_del) {
    dropin_check(eprem_gpu_set_time_step(dropin_run, config.tDel), "time step");
    dropin_t_del = config.tDel;
  }
}

/* grid[] shells 1..N of every stream <-> nodes[field][s*N+k] (k = shell-1) */
static void dropin_pack_nodes(uint64_t mask) {
  const int N = TOTAL_NUM_SHELLS;
  for (size_t s = 0; s < (size_t)NUM_STREAMS; s++)
    for (int k = 0; k < N; k++) {
      Node_t *n = &grid[s * LOCAL_NUM_SHELLS + k + 1];
      for (int fld = 0; fld < EPREM_NODE_NFIELDS; fld++)
        if (mask & EPREM_NODE_MASK(fld))
          dropin_nodes[fld * dropin_sn + s * N + k] = *dropin_member(n, fld);
    }
}

static void dropin_unpack_nodes(uint64_t mask) {
  const int N = TOTAL_NUM_SHELLS;
  for (size_t s = 0; s < (size_t)NUM_STREAMS; s++)
    for (int k = 0; k < N; k++) {
      Node_t *n = &grid[s * LOCAL_NUM_SHELLS + k + 1];
      for (int fld = 0; fld < EPREM_NODE_NFIELDS; fld++)
        if (mask & EPREM_NODE_MASK(fld))
          *dropin_member(n, fld) = dropin_nodes[fld * dropin_sn + s * N + k];
    }
}

#define DROPIN_EP_IN                                                                     \
  (EPREM_NODE_MASK(EPREM_NODE_RX) | EPREM_NODE_MASK(EPREM_NODE_RY) |                    \
   EPREM_NODE_MASK(EPREM_NODE_RZ) | EPREM_NODE_MASK(EPREM_NODE_RMAG) |                  \
   EPREM_NODE_MASK(EPREM_NODE_BMAG) | EPREM_NODE_MASK(EPREM_NODE_DLNB) |                \
   EPREM_NODE_MASK(EPREM_NODE_DLNN) | EPREM_NODE_MASK(EPREM_NODE_DUPAR))
/* and, with shell diffusion, the direction of B (ShellData) */
#define DROPIN_SHELL_IN                                                                  \
  (EPREM_NODE_MASK(EPREM_NODE_BVEC_X) | EPREM_NODE_MASK(EPREM_NODE_BVEC_Y) |            \
   EPREM_NODE_MASK(EPREM_NODE_BVEC_Z))
#define DROPIN_EP_OUT                                                                    \
  (EPREM_NODE_MASK(EPREM_NODE_DS) | EPREM_NODE_MASK(EPREM_NODE_BMAG_PLUS) |             \
   EPREM_NODE_MASK(EPREM_NODE_BMAG_MINUS))

/* f between eParts (shells 1..N of each stream, pitch SSPEM past the
 * INNER_SHELL row, src/global.h:61) and the device */
static void dropin_f_to_device(void) {
  if (dropin_f_dev) return;
  dropin_check(eprem_gpu_upload_f_pitched(dropin_run, eParts + SPEM, (size_t)SSPEM), "upload f");
  dropin_f_dev = 1;
  dropin_f_stale = 0;
}

static void dropin_f_to_host(void) {
  if (!dropin_f_stale) return;
  dropin_f_stale = 0;
  dropin_check(eprem_gpu_download_f_pitched(dropin_run, eParts + SPEM, (size_t)SSPEM),
               "download f");
}

/* useShellDiffusion / useDrift: hand the run the NEWS links gridStructInit
 * gave every shell (initNEWS + initCopyAll, src/cubeShellInit.c:46-94) as
 * stream indices.  The driver's first updateMhd comes before gridStructInit
 * (src/eprem.c:470-480), so this waits for the first particle update.  The
 * run forms ShellData's lengths itself at each update; the driver's own
 * ShellData call (src/eprem.c:647-650) only fills host fields nothing here
 * reads. */
static int dropin_shell_ready = 0;
static void dropin_shell_setup(void) {
  if (dropin_shell_ready || (config.useShellDiffusion <= 0 && config.useDrift <= 0)) return;
  int32_t *news = (int32_t *)malloc(sizeof(int32_t) * 4 * (size_t)NUM_STREAMS);
  if (!news) panic("GPU path: allocation failed");
  for (Index_t face = 0; face < NUM_FACES; face++)
    for (Index_t row = 0; row < FACE_ROWS; row++)
      for (Index_t col = 0; col < FACE_COLS; col++) {
        const Node_t *nd = &grid[idx_frcs(face, row, col, INNER_ACTIVE_SHELL)];
        const Neighbor_t *nb[4] = {&nd->n, &nd->e, &nd->w, &nd->s};
        const size_t s = ((size_t)face * FACE_ROWS + row) * FACE_COLS + col;
        for (int k = 0; k < 4; k++)
          news[s * 4 + k] = (int32_t)((nb[k]->face * FACE_ROWS + nb[k]->row) * FACE_COLS + nb[k]->col);
      }
  if (config.useShellDiffusion > 0)
    dropin_check(eprem_gpu_set_shell_diffusion(dropin_run, news, config.kperxkpar),
                 "shell diffusion");
  if (config.useDrift > 0) {
    eprem_drift_params_t dp;
    dp.lnpmin = lnpmin;
    dp.charge = config.charge[0];
    dp.mass = config.mass[0];
    dropin_check(eprem_gpu_set_drift(dropin_run, news, &dp), "drift");
  }
  free(news);
  dropin_shell_ready = 1;
}

void updateEnergeticParticles(void) {
  dropin_init();
  dropin_sync_step();
  dropin_shell_setup();
  double t0 = MPI_Wtime();
  dropin_f_to_device();
  const uint64_t in = DROPIN_EP_IN | (config.useShellDiffusion > 0 ? DROPIN_SHELL_IN : 0);
  dropin_pack_nodes(in);
  dropin_check(eprem_gpu_upload_nodes(dropin_run, dropin_nodes, in), "upload nodes");
  dropin_check(eprem_gpu_update_energetic_particles(dropin_run, t_global),
               "updateEnergeticParticles");
  dropin_f_stale = 1;
  eprem_ep_stats_t st;
  dropin_check(eprem_gpu_read_stats(dropin_run, &st), "updateEnergeticParticles");
  dropin_check(eprem_gpu_download_nodes(dropin_run, dropin_nodes, DROPIN_EP_OUT),
               "download nodes");
  dropin_unpack_nodes(DROPIN_EP_OUT);
  /* the driver's per-step report (src/eprem.c:694-716) */
  if (st.max_subcycles_change > maxsubcycles_energychange)
    maxsubcycles_energychange = st.max_subcycles_change;
  if (st.max_subcycles_focusing > maxsubcycles_focusing)
    maxsubcycles_focusing = st.max_subcycles_focusing;
  if (st.min_tau < min_tau) min_tau = st.min_tau;
  timer_diffusestream += MPI_Wtime() - t0;
}

/* rotSunAndSpawnShell for one rank (no shell arrives from an inner rank,
 * src/simCore.c:481-599): rotate the sun, ripple the shells out -- the nodes
 * on the host as rippleShellsOut does (src/simCore.c:700-735: each node takes
 * its inner neighbour's data but keeps its own neighbour links), f on the
 * device with the INNER_SHELL rows as the new first shell -- and spawn the
 * new shell's positions with the reference's own spawnNewShell. */
void rotSunAndSpawnShell(Time_t t_sun_del) {
  dropin_init();
  azi_sun += (config.omegaSun * t_sun_del);
  if (azi_sun > PI) azi_sun -= TWO_PI;
  for (size_t s = 0; s < (size_t)NUM_STREAMS; s++)
    for (Index_t shell = OUTER_SHELL; shell > INNER_SHELL; shell--) {
      Node_t *dst = &grid[s * LOCAL_NUM_SHELLS + shell];
      const Neighbor_t n = dst->n, e = dst->e, w = dst->w, so = dst->s;
      const Neighbor_t in = dst->streamIn, out = dst->streamOut;
      *dst = *(dst - 1);
      dst->n = n;
      dst->e = e;
      dst->w = w;
      dst->s = so;
      dst->streamIn = in;
      dst->streamOut = out;
    }
  dropin_f_to_device();
  dropin_check(eprem_gpu_ripple_f(dropin_run, eParts, (size_t)SSPEM), "rotSunAndSpawnShell");
  dropin_f_stale = 1;
  spawnNewShell();
}

/* Whether dataDumpIO (src/unifiedOutput.c:1479-1531) writes anything at
 * this time, by its own conditions. */
static int dropin_output_due(void) {
  const double t = t_global * DAY;
  return (config.unifiedOutput > 0 && t >= config.unifiedOutputTime) ||
         (config.numObservers > 0 && t >= config.pointObserverOutputTime) ||
         (config.epremDomain > 0 && t >= config.epremDomainOutputTime) ||
         (config.unstructuredDomain > 0 && t >= config.epremDomainOutputTime);
}

/* streamFluxOutput = 1 with no other output that reads eParts: the observer
 * files take the omnidirectional flux alone, which computeFlux
 * (src/unifiedOutput.c:153-180) forms from each row's mu-average of f.  The
 * device's flux (S*N*E values, 1/M of f) comes down instead of f, and each
 * eParts row of the output is set to its mu-average J / (2E) -- all that
 * computeFlux reads of it.  eParts stays marked as older than the device's
 * f, so any later reader of the whole of f still brings it down. */
static double *dropin_flux = NULL;
static int dropin_flux_only(void) {
  return config.streamFluxOutput == 1 && config.numObservers == 0 && config.epremDomain == 0 &&
         config.unstructuredDomain == 0;
}

static void dropin_flux_to_host(void) {
  const size_t N = TOTAL_NUM_SHELLS, E = NUM_ESTEPS, M = NUM_MUSTEPS;
  if (!dropin_flux) {
    dropin_flux = (double *)eprem_gpu_host_alloc(sizeof(double) * dropin_sn * E);
    if (!dropin_flux) panic("GPU path: host flux buffer allocation failed");
  }
  dropin_check(eprem_gpu_omni_flux(dropin_run, dropin_flux), "omnidirectional flux");
  for (size_t s = 0; s < (size_t)NUM_STREAMS; s++)
    for (size_t k = 0; k < N; k++) {
      Scalar_t *row = eParts + SPEM + s * SSPEM + k * E * M;
      const double *j = dropin_flux + (s * N + k) * E;
      for (size_t e = 0; e < E; e++) {
        const Scalar_t iso = j[e] / (2.0 * egrid[e]);
        for (size_t m = 0; m < M; m++) row[e * M + m] = iso;
      }
    }
}

/* The driver's output reads eParts: bring it up to date first (when the
 * output is due at all; the driver calls dataDumpIO every step). */
void dataDumpIO(void) {
  if (dropin_run && dropin_f_stale && dropin_output_due()) {
    if (dropin_flux_only())
      dropin_flux_to_host();
    else
      dropin_f_to_host();
  }
  dataDumpIO_cpu();
}

/* The driver sets eParts to the seed population: eParts is the current f
 * from here on, the device's copy is taken again at its next use. */
void initEnergeticParticles(void) {
  initEnergeticParticles_cpu();
  dropin_f_dev = 0;
  dropin_f_stale = 0;
}

/* ---- MAS background --------------------------------------------------- */
static int dropin_mas_ready = 0;
static Index_t dropin_mas_file[2] = {-1, -1};

/* The reference's slot globals (src/readMAS.h) as an ABI slice. */
#define DROPIN_MAS_FIELD(S, i, F, SL)                                  \
  do {                                                                 \
    (S)->data[i] = mas##F##_##SL;                                      \
    (S)->mesh[i][0] = mas##F##rDim_##SL;                               \
    (S)->mesh[i][1] = mas##F##tDim_##SL;                               \
    (S)->mesh[i][2] = mas##F##pDim_##SL;                               \
    (S)->dims[i][0] = mas##F##rDimMax_##SL[0];                         \
    (S)->dims[i][1] = mas##F##tDimMax_##SL[0];                         \
    (S)->dims[i][2] = mas##F##pDimMax_##SL[0];                         \
  } while (0)

static void dropin_mas_slot(int slot, eprem_mas_slice_t *sl) {
  if (slot == 0) {
    DROPIN_MAS_FIELD(sl, 0, Bp, 0); DROPIN_MAS_FIELD(sl, 1, Bt, 0); DROPIN_MAS_FIELD(sl, 2, Br, 0);
    DROPIN_MAS_FIELD(sl, 3, Vp, 0); DROPIN_MAS_FIELD(sl, 4, Vt, 0); DROPIN_MAS_FIELD(sl, 5, Vr, 0);
    DROPIN_MAS_FIELD(sl, 6, D, 0);
  } else {
    DROPIN_MAS_FIELD(sl, 0, Bp, 1); DROPIN_MAS_FIELD(sl, 1, Bt, 1); DROPIN_MAS_FIELD(sl, 2, Br, 1);
    DROPIN_MAS_FIELD(sl, 3, Vp, 1); DROPIN_MAS_FIELD(sl, 4, Vt, 1); DROPIN_MAS_FIELD(sl, 5, Vr, 1);
    DROPIN_MAS_FIELD(sl, 6, D, 1);
  }
}

/* Bring the device slots up to the slices masGetInterpData has loaded. */
static void dropin_mas_sync(void) {
  if (!dropin_mas_ready) {
    eprem_mas_params_t mp;
    memset(&mp, 0, sizeof(mp));
    mp.radial_max = config.masRadialMax;
    mp.v_min = config.masVmin;
    mp.cor_rotate_fake = config.masCorRotateFake;
    mp.rotate_solution = config.masRotateSolution;
    mp.max_slices = 2;
    dropin_check(eprem_gpu_mas_init(dropin_run, &mp), "MAS set-up");
    dropin_mas_ready = 1;
  }
  const Index_t idx[2] = {masFileIndex0, masFileIndex1};
  for (int slot = 0; slot < 2; slot++)
    if (idx[slot] != dropin_mas_file[slot]) {
      eprem_mas_slice_t sl;
      dropin_mas_slot(slot, &sl);
      dropin_check(eprem_gpu_mas_load_slice(dropin_run, slot, &sl), "MAS slice upload");
      dropin_mas_file[slot] = idx[slot];
    }
  dropin_check(eprem_gpu_mas_select(dropin_run, 0, 1, s_cor, phiOffset), "MAS slices");
}

void updateMhd(void) {
  dropin_init();
  dropin_sync_step();
  const uint64_t all = EPREM_NODE_MASK_ALL;
  if (mhdGridStatus == MHD_MAS && config.useDrift > 0)
    panic("GPU path: drift with the MAS background is not supported by this build");
  if (mhdGridStatus == MHD_MAS) {
    dropin_mas_sync();
    dropin_check(eprem_gpu_mas_use(dropin_run, 1), "updateMhd");
  } else if (dropin_mas_ready) {
    dropin_check(eprem_gpu_mas_use(dropin_run, 0), "updateMhd");
  }
  dropin_pack_nodes(all);
  dropin_check(eprem_gpu_upload_nodes(dropin_run, dropin_nodes, all), "upload nodes");
  dropin_check(eprem_gpu_update_mhd(dropin_run, t_global), "updateMhd");
  dropin_check(eprem_gpu_download_nodes(dropin_run, dropin_nodes, all), "download nodes");
  dropin_unpack_nodes(all);
}

void moveNodes(Scalar_t dt) {
  dropin_init();
  dropin_sync_step();
  const uint64_t mv = EPREM_NODE_MASK(EPREM_NODE_RX) | EPREM_NODE_MASK(EPREM_NODE_RY) |
                      EPREM_NODE_MASK(EPREM_NODE_RZ) | EPREM_NODE_MASK(EPREM_NODE_RMAG) |
                      EPREM_NODE_MASK(EPREM_NODE_VVEC_X) | EPREM_NODE_MASK(EPREM_NODE_VVEC_Y) |
                      EPREM_NODE_MASK(EPREM_NODE_VVEC_Z) | EPREM_NODE_MASK(EPREM_NODE_ROLD_X) |
                      EPREM_NODE_MASK(EPREM_NODE_ROLD_Y) | EPREM_NODE_MASK(EPREM_NODE_ROLD_Z);
  dropin_pack_nodes(mv);
  dropin_check(eprem_gpu_upload_nodes(dropin_run, dropin_nodes, mv), "upload nodes");
  dropin_check(eprem_gpu_move_nodes(dropin_run, dt), "moveNodes");
  dropin_check(eprem_gpu_download_nodes(dropin_run, dropin_nodes, mv), "download nodes");
  dropin_unpack_nodes(mv);
}

void masMoveNodes(Scalar_t dt) {
  dropin_init();
  dropin_sync_step();
  dropin_mas_sync();
  const uint64_t all = EPREM_NODE_MASK_ALL;
  dropin_pack_nodes(all);
  dropin_check(eprem_gpu_upload_nodes(dropin_run, dropin_nodes, all), "upload nodes");
  dropin_check(eprem_gpu_mas_move_nodes(dropin_run, dt), "masMoveNodes");
  dropin_check(eprem_gpu_download_nodes(dropin_run, dropin_nodes, all), "download nodes");
  dropin_unpack_nodes(all);
}
