/*
 * eprem_gpu.h -- C ABI of the GB300 (sm_103a) implementation of EPREM's
 * per-timestep energetic-particle update.
 *
 * The reference (predsci/eprem) keeps all state in C globals and exposes the
 * hot path as four argument-less entry points called from its driver loop
 * (src/eprem.c:620-671):
 *
 *   void updateEnergeticParticles(void);   src/energeticParticles.h:51
 *   void updateMhd(void);                  src/flow.h:45
 *   void moveNodes(Scalar_t dt);           src/simCore.h:71
 *   void masMoveNodes(Scalar_t dt);        src/masInterp.h:186
 *
 * This library replaces their bodies.  A host shim (eprem_gb300/host/
 * eprem_dropin.c) keeps those four symbols, packs the reference globals
 * (grid[], eParts[], config, egrid/vgrid/...) into the plain arrays below and
 * calls the functions of this header.  Nothing here uses C++ or torch types:
 * plain pointers, sizes and status codes only.
 *
 * State lives on the device inside an opaque run handle.  Every stream of the
 * cube-sphere grid is held by one GPU (the reference spreads the nodes of each
 * stream over MPI ranks, src/mpiInit.c:91-147).
 *
 * Layouts (host and device alike):
 *   f      [stream][node][energy][mu], mu fastest.  For one MPI rank this is
 *          the reference eParts layout idx_frcsspem (src/global.h:61) with the
 *          INNER_SHELL ghost (shell 0) removed: node k is shell k+1, stream
 *          index s = face*ROWS*COLS + row*COLS + col (computeLines order,
 *          src/unifiedOutput.c:64-92).
 *   nodes  [field][stream*num_nodes + node], one double per Node_t member
 *          used by the hot path (src/cubeShellStruct.h:51-93), fields
 *          enumerated by eprem_node_field below.
 *
 * All functions return EPREM_GPU_OK (0) or a negative status; the message of
 * the last failure on the calling thread is available from
 * eprem_gpu_last_error().  No exception crosses this boundary.  The library is
 * not re-entrant for one run handle (the reference is single-threaded per
 * rank, MPI_THREAD_FUNNELED, src/mpiInit.c:57).
 */
#ifndef EPREM_GPU_H
#define EPREM_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define EPREM_GPU_OK               0
#define EPREM_GPU_ERR_ARG         -1  /* bad argument or unsupported size      */
#define EPREM_GPU_ERR_CUDA        -2  /* CUDA runtime failure                   */
#define EPREM_GPU_ERR_NAN         -3  /* NaN in f   (reference checkNaN->panic) */
#define EPREM_GPU_ERR_INF         -4  /* Inf in f   (reference checkInf->panic) */
#define EPREM_GPU_ERR_DS          -5  /* ds <= 0 (FindSegmentLengths panic)     */
#define EPREM_GPU_ERR_SUBCYCLES   -6  /* sub-cycle count above params cap       */
#define EPREM_GPU_ERR_UNSUPPORTED -7  /* option the reference path does not have
                                         or that this library does not build   */
#define EPREM_GPU_ERR_STATE       -8  /* stream thinned to fewer than 3 nodes   */

/* ---- arithmetic forms -------------------------------------------------- */
#define EPREM_FP64 0  /* plain form: every operation in IEEE double          */
#define EPREM_FP32 1  /* f and the stencil/scattering arithmetic in float;
                         positions, distances, dt/CFL reductions and
                         conservation sums in double.  The device holds
                         f * 2^64 (uploads, downloads and fluxes convert), so
                         f values between 6.4e-58 and 1.8e19 are held as
                         normal floats; smaller ones floor at 6.4e-58       */

/* ---- sizes -------------------------------------------------------------- */
typedef struct {
  int32_t num_streams;   /* NUM_STREAMS = 6*numRowsPerFace*numColumnsPerFace */
  int32_t num_nodes;     /* numNodesPerStream (TOTAL_NUM_SHELLS), >= 3       */
  int32_t num_species;   /* numSpecies; must be 1 (see DESIGN notes)         */
  int32_t num_energies;  /* numEnergySteps, 2..64                            */
  int32_t num_mu;        /* numMuSteps, 2..64                                */
  int32_t precision;     /* EPREM_FP64 or EPREM_FP32                         */
} eprem_dims_t;

/* ---- run parameters: the config members the hot path reads -------------
 * Values are the reference's after setRuntimeConstants()
 * (src/configuration.c:325-348): times in AU/c, speeds in c, densities in
 * MHD_DENSITY_NORM, fields in MHD_B_NORM. */
typedef struct {
  double  r_scale;                  /* config.rScale                          */
  double  t_del;                    /* config.tDel (AU/c)                     */
  int32_t num_ep_steps;             /* config.numEpSteps                      */
  int32_t use_parallel_diffusion;   /* config.useParallelDiffusion            */
  int32_t use_adiabatic_focus;      /* config.useAdiabaticFocus               */
  int32_t use_adiabatic_change;     /* config.useAdiabaticChange              */
  int32_t check_seed_population;    /* config.checkSeedPopulation             */
  int32_t use_ep_boundary;          /* config.useEPBoundary                   */
  int32_t use_boundary_function;    /* config.useBoundaryFunction             */
  int32_t adiabatic_focus_alg;      /* 1 Euler upwind, 2 RK3 upwind, 3 RK3+WENO3 */
  int32_t adiabatic_change_alg;     /* same                                   */
  double  damp_cooling;             /* config.dampCooling                     */
  double  dsh_min;                  /* config.dsh_min (AU)                    */
  int32_t mfp_type;                 /* 1: r-scaled, 2: B-scaled               */
  double  lamo;                     /* config.lamo (AU)                       */
  double  mfp_radial_power;         /* config.mfpRadialPower                  */
  double  mfp_b_power;              /* config.mfpBPower                       */
  double  mhd_bs_au;                /* config.mhdBsAu                         */
  double  bf_amplitude;             /* config.boundaryFunctAmplitude          */
  double  bf_xi;                    /* config.boundaryFunctXi                 */
  double  bf_gamma;                 /* config.boundaryFunctGamma              */
  double  bf_beta;                  /* config.boundaryFunctBeta               */
  double  bf_ecutoff;               /* config.boundaryFunctEcutoff (MeV)      */
  double  bf_r0;                    /* config.boundaryFunctR0 (AU)            */
  /* analytic background (src/flow.c), used by eprem_gpu_update_mhd */
  double  mhd_us;                   /* config.mhdUs   (flowMag/C)             */
  double  mhd_ns_au;                /* config.mhdNsAu                         */
  double  omega_sun;                /* config.omegaSun                        */
  int32_t ideal_shock;              /* config.idealShock                      */
  double  ideal_shock_sharpness;
  double  ideal_shock_scale_length;
  double  ideal_shock_jump;
  double  ideal_shock_falloff;
  double  ideal_shock_speed;        /* cm/s, as in the config file           */
  double  ideal_shock_init_time;    /* days, as in the config file           */
  double  ideal_shock_theta;
  double  ideal_shock_phi;
  double  ideal_shock_width;
  int32_t max_subcycles;            /* cap on any sub-cycle count; above it the
                                       update stops with ERR_SUBCYCLES (0 means
                                       1,000,000).  The reference has no cap. */
  int32_t stream_variant;           /* streaming-kernel shape in the FP32 form
                                       (tuning; results agree to rounding):
                                       kind + 8 * shape.  kind 0 automatic
                                       (the first of 7, 5, 4, 3 that fits);
                                       3 several nodes per thread; 4 as 3
                                       with packed fp32x2 arithmetic; 5 as 4
                                       with compile-time cell guards (M = 8,
                                       16, ..., 64 and m0 = M/2); 6 and 7 as
                                       5 with the mu < 0 half in mirror
                                       order, one upwind coefficient per two
                                       cells (M = 20 or 40 and the seed
                                       boundary on; 7 with the coefficients in shared
                                       memory and, on one CTA per stream,
                                       no CTA barrier per sub-cycle).  shape 0
                                       automatic, k >= 1 the k-th CTA shape
                                       (threads, nodes per thread, cluster)
                                       of the run's mu bin.  A shape whose
                                       stream needs a cluster of more than
                                       8 CTAs is refused.                  */
} eprem_params_t;

/* ---- 1-D grids built by initEnergeticParticlesGrids
 *      (src/energeticParticlesInit.c:36-100); host pointers, copied at create */
typedef struct {
  const double *egrid;     /* [E] kinetic energy / (mp c^2)                   */
  const double *vgrid;     /* [E] speed / c                                   */
  const double *vgrid_i;   /* [E] 1 / vgrid                                   */
  const double *mugrid;    /* [M] mu cell centres                             */
  const double *rigidity;  /* [E] rigidity^rigidityPower (species 0)          */
  double dlnp;             /* ln p spacing                                    */
  double dmu;              /* mu spacing                                      */
} eprem_grids_t;

/* ---- per-node fields (Node_t members, src/cubeShellStruct.h:51-93) ------- */
enum eprem_node_field {
  EPREM_NODE_RX = 0, EPREM_NODE_RY, EPREM_NODE_RZ, /* r (units of rScale)     */
  EPREM_NODE_RMAG,                                 /* rmag                    */
  EPREM_NODE_BMAG,                                 /* mhdBmag                 */
  EPREM_NODE_DLNB,                                 /* mhdDlnB                 */
  EPREM_NODE_DLNN,                                 /* mhdDlnN                 */
  EPREM_NODE_DUPAR,                                /* mhdDuPar                */
  EPREM_NODE_DS,                                   /* ds          (output)    */
  EPREM_NODE_BMAG_PLUS,                            /* mhdBmagPlus (output)    */
  EPREM_NODE_BMAG_MINUS,                           /* mhdBmagMinus (output)   */
  EPREM_NODE_BR, EPREM_NODE_BTHETA, EPREM_NODE_BPHI,
  EPREM_NODE_VR, EPREM_NODE_VTHETA, EPREM_NODE_VPHI,
  EPREM_NODE_VMAG,
  EPREM_NODE_DENSITY,
  EPREM_NODE_DIVV,
  EPREM_NODE_BVEC_X, EPREM_NODE_BVEC_Y, EPREM_NODE_BVEC_Z,
  EPREM_NODE_VVEC_X, EPREM_NODE_VVEC_Y, EPREM_NODE_VVEC_Z,
  EPREM_NODE_BMAG_OLD,
  EPREM_NODE_DENSITY_OLD,
  EPREM_NODE_VSPH_OLD_R, EPREM_NODE_VSPH_OLD_THETA, EPREM_NODE_VSPH_OLD_PHI,
  EPREM_NODE_DS_OLD,
  EPREM_NODE_ROLD_X, EPREM_NODE_ROLD_Y, EPREM_NODE_ROLD_Z,
  EPREM_NODE_ROLDER_X, EPREM_NODE_ROLDER_Y, EPREM_NODE_ROLDER_Z,
  EPREM_NODE_NFIELDS
};
#define EPREM_NODE_MASK(field) (1ull << (field))
#define EPREM_NODE_MASK_ALL ((1ull << EPREM_NODE_NFIELDS) - 1ull)

/* ---- per-call statistics (the driver's log line, src/eprem.c:694-716) ---- */
typedef struct {
  int32_t max_subcycles_change;    /* maxsubcycles_energychange                */
  int32_t max_subcycles_focusing;  /* maxsubcycles_focusing                    */
  int32_t max_substeps_stream;     /* largest DiffuseStreamData nsteps         */
  int32_t pad;
  double  min_tau;                 /* min_tau (DBL_MAX when nothing computed)  */
  double  stream_cell_subcycles;   /* sum over (stream, E) of nsteps*list*mu   */
  double  focus_cell_subcycles;    /* sum over nodes of N_sub*E*mu (focusing)  */
  double  change_cell_subcycles;   /* sum over nodes of N_sub*E*mu (change)    */
} eprem_ep_stats_t;

/* Kernel kinds for the optional per-launch timing below. */
enum eprem_kernel_kind {
  EPREM_KERNEL_GEOMETRY = 0,  /* updateStreamValues, GetStreamList, node factors */
  EPREM_KERNEL_STREAM,        /* DiffuseStreamData (+ seed check)               */
  EPREM_KERNEL_NODE,          /* AdiabaticFocusing + AdiabaticChange            */
  EPREM_KERNEL_SEED_CHECK,    /* seedPopulationCheck alone                      */
  EPREM_KERNEL_MHD,           /* updateMhd                                      */
  EPREM_KERNEL_MOVE,          /* moveNodes                                      */
  EPREM_KERNEL_FLUX,          /* omnidirectional flux                           */
  EPREM_KERNEL_CONVERT,       /* f format conversion (FP32 form)                */
  EPREM_KERNEL_SHELL,         /* ShellData + DiffuseShellData                   */
  EPREM_KERNEL_NKINDS
};
typedef struct {
  int32_t launches;   /* launches of this kind since the last read */
  int32_t pad;
  double  total_ms;   /* summed CUDA-event time of those launches  */
} eprem_kernel_time_t;

typedef struct eprem_gpu_run eprem_gpu_run;

/* Create a run on the current CUDA device and allocate its device state.
 * No counterpart in the reference beyond allocateGlobalVariables()
 * (src/global.c:80-132) and initMPI_energeticParticlesTypes()
 * (src/energeticParticlesTypes.c:38-69), which size the same arrays. */
int eprem_gpu_create(const eprem_dims_t *dims, const eprem_params_t *params,
                     const eprem_grids_t *grids, eprem_gpu_run **out);
int eprem_gpu_destroy(eprem_gpu_run *run);

/* f: S*N*E*M doubles from/to host memory (stream-major, mu fastest).
 * Replaces the MPI gather/scatter of eParts (src/simCore.c:178-318); in the
 * FP32 form the device copy is float and these convert. */
int eprem_gpu_upload_f(eprem_gpu_run *run, const double *f_host);
int eprem_gpu_download_f(eprem_gpu_run *run, double *f_host);

/* The same with stream s's N*E*M values at f + s * stream_pitch (0: N*E*M):
 * the reference's eParts + SPEM with pitch SSPEM (src/global.h:61) directly,
 * as the drop-in moves f only when the driver reads or writes it there. */
int eprem_gpu_upload_f_pitched(eprem_gpu_run *run, const double *f_host, size_t stream_pitch);
int eprem_gpu_download_f_pitched(eprem_gpu_run *run, double *f_host, size_t stream_pitch);

/* rippleShellsOut (src/simCore.c:700-735) for f, on the device: node k of
 * every stream takes node k-1's values (the outermost node's are dropped)
 * and node 0 takes the stream's template row, E*M doubles at
 * tmpl_host + s * stream_pitch (0: E*M) -- the reference's INNER_SHELL, so
 * eParts with pitch SSPEM.  With it the drop-in keeps f on the device from
 * step to step: rotSunAndSpawnShell (src/simCore.c:443-630) ripples it there
 * instead of moving all of eParts on the host. */
int eprem_gpu_ripple_f(eprem_gpu_run *run, const double *tmpl_host, size_t stream_pitch);

/* nodes: EPREM_NODE_NFIELDS*S*N doubles, [field][stream*N+node]; only the
 * fields whose bit is set in field_mask are copied. */
int eprem_gpu_upload_nodes(eprem_gpu_run *run, const double *nodes_host,
                           uint64_t field_mask);
int eprem_gpu_download_nodes(eprem_gpu_run *run, double *nodes_host,
                             uint64_t field_mask);

/* One call of updateEnergeticParticles() (src/energeticParticles.c:70-203):
 * numEpSteps operator-split sub-steps of streaming + isotropisation
 * (DiffuseStreamData :2240-2490), adiabatic focusing (:1537-1803) and
 * adiabatic change (:808-1077), with updateStreamValues
 * (src/simCore.c:326-435), seedPopulationCheck
 * (src/energeticParticlesBoundary.c:28-59) and GetStreamList /
 * FindSegmentLengths (:2150-2234, :2496-2601).  Asynchronous on the run's
 * stream; device-side failures (NaN, Inf, ds<=0, cap) are reported by the
 * next eprem_gpu_synchronize / read_stats / download call.  t_global is
 * accepted for interface fidelity; the MAS-heliospheric switches that read it
 * are not supported. */
int eprem_gpu_update_energetic_particles(eprem_gpu_run *run, double t_global);

/* The same update with f in host memory: stream s's N*E*M values start at
 * f_in + s * stream_pitch (and f_out + s * stream_pitch); stream_pitch 0
 * means N*E*M (f stream-major and contiguous, as eprem_gpu_upload_f); the
 * reference's own array is eParts + SPEM with pitch SSPEM (one INNER_SHELL
 * row before each stream's shells, src/global.h:61, src/global.c:112), so a
 * caller holding f there packs nothing on the host.  (The drop-in keeps f on
 * the device across steps instead: eprem_gpu_ripple_f.)  f_in and f_out may
 * be the same array.  The streams go through in chunks (a short first and last
 * one around six long ones), and each chunk's host-to-device copy, update
 * and device-to-host copy overlap the neighbouring chunks' work, so the
 * copies hide behind the update when the host memory is page-locked
 * (eprem_gpu_host_alloc, or eprem_gpu_host_register on an existing
 * allocation).  Node fields are not copied: upload and download them as for
 * eprem_gpu_update_energetic_particles.  Returns when f_out holds the
 * result; statistics accumulate as for that call.  No reference counterpart
 * beyond the gather / update / scatter of src/simCore.c:178-318 and
 * src/energeticParticles.c:70-203. */
int eprem_gpu_update_energetic_particles_host(eprem_gpu_run *run, const double *f_in,
                                              double *f_out, size_t stream_pitch,
                                              double t_global);

/* Page-locked host memory (NULL on failure) for the host arrays of the calls
 * above: copies from it run asynchronously at the link's rate, which the
 * overlap of eprem_gpu_update_energetic_particles_host needs.  Replaces the
 * malloc of the host staging a caller would otherwise use. */
void *eprem_gpu_host_alloc(size_t bytes);
void eprem_gpu_host_free(void *ptr);
/* Page-lock an existing host allocation in place (cudaHostRegister), e.g.
 * the reference's eParts; EPREM_GPU_ERR_CUDA if the memory cannot be locked
 * (copies from it then stay correct but do not overlap). */
int eprem_gpu_host_register(void *ptr, size_t bytes);
int eprem_gpu_host_unregister(void *ptr);

/* Statistics accumulated since the previous read (then reset), as the driver
 * prints and resets them once per step (src/eprem.c:694-716).  Synchronizes. */
int eprem_gpu_read_stats(eprem_gpu_run *run, eprem_ep_stats_t *stats);

/* updateMhd() for the analytic Parker background, with the ideal shock
 * (src/flow.c:36-154, 241-403, 623-651). */
int eprem_gpu_update_mhd(eprem_gpu_run *run, double t_global);

/* moveNodes(dt): Euler push of every node but the innermost of each stream by
 * the node's flow velocity (src/simCore.c:737-785, delrFlow src/flow.c:162-196). */
int eprem_gpu_move_nodes(eprem_gpu_run *run, double dt);

/* The step length config.tDel (AU/c), which MAS-coupled runs change between
 * steps: SetDT (src/simCore.c:800-880) sets it to the spacing of the MAS
 * slice times around t_global.  It sets the EP sub-step dt = t_del /
 * numEpSteps (src/energeticParticles.c:99) and the time scale of the
 * background's divV.  Takes effect from the next call; an ensemble captured
 * before the change keeps the step it captured (rebuild it).  t_del must be
 * finite and > 0. */
int eprem_gpu_set_time_step(eprem_gpu_run *run, double t_del);

/* Cross-field (shell) diffusion: config.useShellDiffusion = 1 with
 * config.kperxkpar (src/configuration.c:77, :124).  Every later
 * eprem_gpu_update_energetic_particles then runs DiffuseShellData
 * (src/energeticParticles.c:419-554) after each sub-step's streaming,
 * focusing and change of all streams (:178-182), with the perpendicular
 * neighbour lengths of ShellData (:254-413) formed at the start of the call
 * from the node positions and B, as the driver calls ShellData right before
 * the update (src/eprem.c:647-671).  news: num_streams*4 stream indices
 * (face*R*C + row*C + col) of each stream's north, east, west and south
 * neighbour on its shell -- the Node_t links n, e, w, s of
 * src/cubeShellStruct.h that initNEWS / initCopyAll set, the same on every
 * shell; NULL switches the diffusion off.  Allocates the gather lists and an
 * f-sized scratch on the first call.  The diffusion couples the streams, so
 * eprem_gpu_update_energetic_particles_host then moves all of f in one copy
 * each way instead of pipelining chunks, and ensembles refuse such runs.
 * EPREM_GPU_ERR_ARG for a neighbour out of range or kperxkpar < 1e-33. */
int eprem_gpu_set_shell_diffusion(eprem_gpu_run *run, const int32_t *news, double kperxkpar);

/* Drift: config.useDrift = 1 (src/configuration.c:126).  The drift velocity
 * of driftVelocity (src/energeticParticles.c:210-246) needs the particles'
 * momentum grid and charge-to-mass ratio, which eprem_params_t does not
 * carry. */
typedef struct {
  double lnpmin;  /* lnpmin (src/energeticParticlesTypes.c): p(E) = exp(lnpmin + E dlnp) */
  double charge;  /* config.charge[0] (units of the proton charge)                     */
  double mass;    /* config.mass[0]   (units of the proton mass)                       */
} eprem_drift_params_t;

/* Switch drift on (dp non-NULL) or off (dp NULL).  While on, every
 * eprem_gpu_update_mhd of the analytic background also forms curl(B)/B^2 at
 * each node (mhdCurlBoverB2 / curlBoverB2, src/flow.c:127-128, :411-616:
 * centred differences of the Parker field, ideal shock included), and once
 * the NEWS links are given (news: as for eprem_gpu_set_shell_diffusion; NULL
 * keeps the links of an earlier call, so the curl can be switched on before
 * the grid's links exist) every eprem_gpu_update_energetic_particles runs
 * DriftShellData (src/energeticParticles.c:561-801) after each sub-step,
 * after the shell diffusion: each node k >= 1 hands
 * min(v_d . e_n rScale / dl * dt / dl, 0.025) of its f to each NEWS
 * neighbour its drift velocity points to (dl: the neighbour distance of
 * ShellData), summed in the reference's order.  The MAS background is
 * refused (EPREM_GPU_ERR_UNSUPPORTED): inside the MAS domain the reference
 * leaves curl(B)/B^2 to masGetNode, which does not form it
 * (src/masInterp.c:941-942).  Drift couples the streams, as the shell
 * diffusion does. */
int eprem_gpu_set_drift(eprem_gpu_run *run, const int32_t *news,
                        const eprem_drift_params_t *dp);

/* Omnidirectional flux J = 2 E <f>_mu per (stream, node, energy), the
 * quantity computeFlux writes (src/unifiedOutput.c:153-180), without its
 * output unit scale.  out: S*N*E doubles, host memory.  Synchronizes. */
int eprem_gpu_omni_flux(eprem_gpu_run *run, double *out_host);

/* Capacity, in doubles, of the fixed device buffer behind
 * eprem_gpu_omni_flux_static: 1,048,576 values (8 MiB), i.e. S*N*E up to
 * that many (96 streams x 1000 nodes x 10 energies fits). */
#define EPREM_GPU_FLUX_STATIC_MAX 1048576

/* The omnidirectional flux of eprem_gpu_omni_flux, computed by the same
 * kernel, but staged in a fixed device buffer, so this call allocates no
 * device or pinned host memory.  No counterpart in the reference: it exists
 * for callers that cannot allocate at output time -- a run set or ensemble
 * that sizes its runs to fill the GPU's memory up front (where the first
 * eprem_gpu_omni_flux call, which allocates its staging buffer then, could
 * fail for lack of memory in the middle of a simulation), or a host program
 * that budgets device memory at start-up and permits no allocation later.
 *   - The buffer (8 MiB) becomes resident on a device when the first run is
 *     created there: eprem_gpu_create looks up its address, with that device
 *     current, before the run allocates anything, and keeps it until the
 *     process exits.  This call itself loads and allocates nothing.
 *   - Call it with the run's device current; another current device is
 *     refused with EPREM_GPU_ERR_ARG.
 *   - S*N*E above EPREM_GPU_FLUX_STATIC_MAX is rejected with
 *     EPREM_GPU_ERR_ARG before anything is launched; use eprem_gpu_omni_flux.
 *   - Nothing in the buffer needs to start at zero: the kernel writes every
 *     one of the S*N*E values before they are copied out.
 *   - There is one buffer per device, shared by all runs on it.  Calls that
 *     overlap in time (two host threads, or two runs on one device) race on
 *     it; serialise them.  One thread making calls one after another is safe,
 *     since each call synchronizes before it returns.
 *   - Kernel timing (eprem_gpu_set_kernel_timing) does not cover this call.
 * out_host: S*N*E doubles, host memory.  Synchronizes. */
int eprem_gpu_omni_flux_static(eprem_gpu_run *run, double *out_host);

/* Wait for all work of the run; returns the first device-side failure. */
int eprem_gpu_synchronize(eprem_gpu_run *run);

/* The cudaStream_t the run launches on (as void*), and how many kernels it has
 * launched since creation.  Measurement helpers without a reference
 * counterpart. */
void    *eprem_gpu_stream(eprem_gpu_run *run);
uint64_t eprem_gpu_kernel_launches(const eprem_gpu_run *run);

/* ---- MAS coupling (src/masInterp.c, src/readMAS.c) ----------------------
 * The reference reads MAS HDF5 slices into float arrays, one per field and
 * time slot (masBp_0 ... masD_1, src/readMAS.h), each on its own staggered
 * (r, theta, phi) mesh, and interpolates them onto the nodes in updateMhd and
 * masMoveNodes.  File reading stays in the reference; these calls take the
 * arrays it read.  Field order is the reference's: */
#define EPREM_MAS_NFIELDS 7  /* Bp, Bt, Br, Vp, Vt, Vr, rho (src/masInterp.c:593-720) */
typedef struct {
  int32_t dims[EPREM_MAS_NFIELDS][3];       /* points along r, theta, phi per field */
  const float *mesh[EPREM_MAS_NFIELDS][3];  /* r (solar radii), theta, phi (rad)     */
  const float *data[EPREM_MAS_NFIELDS];     /* [phi][theta][r], r fastest, MAS units */
} eprem_mas_slice_t;

typedef struct {
  double  radial_max;       /* config.masRadialMax (solar radii)                  */
  double  v_min;            /* config.masVmin (cm/s)                              */
  int32_t cor_rotate_fake;  /* config.masCorRotateFake                            */
  int32_t rotate_solution;  /* config.masRotateSolution                           */
  int32_t max_slices;       /* device slots for time slices (the reference holds
                               two, state0/state1; HBM holds many)                */
  int32_t pad;
} eprem_mas_params_t;

/* Switch the run to the MAS background: updateMhd takes its MHD_MAS branch
 * (masGetNode, src/masInterp.c:31-68, with masTriLinear :539-740 and the
 * Parker extrapolation masWind :1007-1065 outside masRadialMax) and
 * eprem_gpu_mas_move_nodes becomes available (masMoveNodes). */
int eprem_gpu_mas_init(eprem_gpu_run *run, const eprem_mas_params_t *mp);
/* Copy one time slice (all seven fields with their meshes) into device slot
 * `slot`; the replacement of masReadData's H2D side (src/readMAS.c:705-830).
 * Returns once the copies are done.  A slot keeps its device arrays from
 * load to load while the slice's dimensions stay the same, so only a slot's
 * first load (or a change of grid) allocates. */
int eprem_gpu_mas_load_slice(eprem_gpu_run *run, int slot, const eprem_mas_slice_t *slice);
/* The same, queued: masGetInterpData's next slice (src/readMAS.c:645-998)
 * copied on the run's copy stream while the run's stream computes with the
 * selected pair -- the slot must not be one of them (EPREM_GPU_ERR_STATE).
 * The copies start after the last launch that read the slot and the run's
 * stream waits for them when eprem_gpu_mas_select next names the slot.  The
 * slice's host arrays must stay valid and unchanged until then, and should
 * be page-locked (eprem_gpu_host_alloc / eprem_gpu_host_register): from
 * pageable memory the driver stages the copy and the call may block until it
 * has. */
int eprem_gpu_mas_load_slice_async(eprem_gpu_run *run, int slot,
                                   const eprem_mas_slice_t *slice);
/* Interpolate between slots slot0 and slot1 with the time factor s_cor
 * (masGetInterpData, src/readMAS.c:645-998) and the phi offset phiOffset. */
int eprem_gpu_mas_select(eprem_gpu_run *run, int slot0, int slot1, double s_cor,
                         double phi_offset);
/* masMoveNodes(dt): RK4 push of every node but the innermost of each stream
 * through the interpolated MAS velocity (src/masInterp.c:1281-1393). */
int eprem_gpu_mas_move_nodes(eprem_gpu_run *run, double dt);
/* Which background eprem_gpu_update_mhd uses after eprem_gpu_mas_init: the
 * MAS interpolation (use_mas = 1, mhdGridStatus == MHD_MAS) or the analytic
 * wind (0, MHD_DEFAULT: masGetInterpData keeps the analytic background
 * before the first MAS time, src/readMAS.c:667-674).  The slots stay loaded
 * and eprem_gpu_mas_move_nodes keeps using them either way, as
 * masMoveNodes does. */
int eprem_gpu_mas_use(eprem_gpu_run *run, int use_mas);

/* Per-launch CUDA-event timing of the run's kernels on its stream (off by
 * default).  read_kernel_timing fills out[EPREM_KERNEL_NKINDS], synchronizes
 * and restarts the accumulation.  Measurement helpers without a reference
 * counterpart (the reference accumulates MPI_Wtime per phase instead,
 * src/energeticParticles.c:122-172). */
int eprem_gpu_set_kernel_timing(eprem_gpu_run *run, int enable);
int eprem_gpu_read_kernel_timing(eprem_gpu_run *run, eprem_kernel_time_t *out);

/* FMA throughput of the current GPU in TFLOP/s (EPREM_FP64 or EPREM_FP32),
 * measured by a short kernel of independent FMA chains: the ALU roofline the
 * kernels above are held against.  No reference counterpart. */
int eprem_gpu_alu_peak(int precision, double *tflops);

/* ---- Synthetic state, autotuning and ensembles ----------------------------
 * None of these has a counterpart in the reference, which runs one
 * simulation per process, seeds f by spawning shells and has one kernel
 * shape per operator. */

/* f = sepSeedFunction(E, r) (src/energeticParticlesBoundary.c:67-116) times
 * (1 + perturbation U(-1,1)) per (stream, node, energy), isotropic in mu, at
 * the current node positions; U is the top 53 bits of splitmix64(seed) at
 * index (stream*N + node)*E + energy + 1.  Builds large synthetic states on
 * the device without a host copy of f.  Synchronizes. */
int eprem_gpu_init_seed_population(eprem_gpu_run *run, uint64_t seed, double perturbation);

/* Time the streaming-kernel kinds and CTA shapes that fit this run (FP32
 * form: every kind 3 to 7 with every shape of its mu bin, encoded as
 * eprem_params_t.stream_variant) on a scratch copy of its first 96 streams
 * and keep the fastest; *chosen_variant receives it.  The run's f
 * and statistics are not touched.  The FP64 form has one shape.  Allocates
 * and frees scratch; synchronizes. */
int eprem_gpu_autotune(eprem_gpu_run *run, int *chosen_variant);
/* Force a streaming-kernel shape (EPREM_GPU_ERR_ARG if it does not fit). */
int eprem_gpu_set_stream_variant(eprem_gpu_run *run, int variant);
/* The streaming kernel a run of these sizes would launch, without a run or a
 * device: num_nodes, num_mu, m0 (the first mu cell with mugrid >= 0),
 * precision, variant (eprem_params_t.stream_variant) and seed_boundary
 * (useEPBoundary and useBoundaryFunction both on).  out[0..5]: kind (0 the
 * FP64 kernel; 3 to 7 as stream_variant), mu bin, threads per CTA, list
 * nodes per thread (1 for FP64), CTAs per cluster, nodes a cluster holds.
 * EPREM_GPU_ERR_ARG where no kernel fits.  No counterpart in the
 * reference. */
int eprem_gpu_plan_stream(int num_nodes, int num_mu, int m0, int precision, int variant,
                          int seed_boundary, int out[6]);
/* The streaming kernel this run launches, with its shape, e.g.
 * "k_stream2_mirror<40,256,4> cluster 1" (a string owned by the run, valid
 * until its next eprem_gpu_set_stream_variant / autotune / destroy).  No
 * counterpart in the reference (one CPU loop there). */
const char *eprem_gpu_stream_kernel(eprem_gpu_run *run);

/* A set of independent runs (different sizes and parameters allowed, all on
 * the current device, analytic background) stepped together.  The first
 * eprem_gpu_ensemble_step captures one driver step of every run --
 * moveNodes(tDel), updateMhd(t + tDel), updateEnergeticParticles, t += tDel,
 * the order of src/eprem.c:620-671 -- into one CUDA graph (the runs in
 * schedule of eprem_gpu_ensemble_set_chains); each later step
 * is one launch of that graph.  Each run's time t lives
 * on the device (set_time / get_time, zero at creation).  Until
 * eprem_gpu_ensemble_synchronize returns, the member runs must not be used
 * on their own.  Failures inside a step are reported by synchronize, with the
 * first failing run's status. */
typedef struct eprem_gpu_ensemble eprem_gpu_ensemble;
int eprem_gpu_ensemble_create(eprem_gpu_run *const *runs, int num_runs,
                              eprem_gpu_ensemble **out);
int eprem_gpu_ensemble_destroy(eprem_gpu_ensemble *ens);
int eprem_gpu_ensemble_set_time(eprem_gpu_ensemble *ens, const double *t_global);
int eprem_gpu_ensemble_get_time(eprem_gpu_ensemble *ens, double *t_global);
/* Autotune one run per size class (precision, mu bin, cluster shape) and give
 * its choice to the others of the class; chosen_variants (may be NULL)
 * receives one variant per run.  The next step captures a new graph. */
int eprem_gpu_ensemble_autotune(eprem_gpu_ensemble *ens, int *chosen_variants);
/* How the graph orders the runs.  chains < 0 (the default): lock-step --
 * every run's moveNodes, updateMhd and per-call set-up, then EP sub-step by
 * EP sub-step the streaming of all runs, one launch per group of runs that
 * share a packed streaming kernel (mu bin, CTA shape, cluster size), its
 * (run, stream, energy) slabs ordered longest first by their estimated
 * sub-cycle work so small runs fill the tails of large ones, then each run's
 * node phase (needs the same numEpSteps in every run; otherwise one chain).
 * chains >= 1: that many serial chains side by side, each run's whole step
 * in sequence, runs spread over the chains largest first; 0: one branch per
 * run.  Results are the runs' own in every schedule, bit for bit.  The next
 * step captures a new graph. */
int eprem_gpu_ensemble_set_chains(eprem_gpu_ensemble *ens, int chains);
int eprem_gpu_ensemble_step(eprem_gpu_ensemble *ens);
int eprem_gpu_ensemble_synchronize(eprem_gpu_ensemble *ens);
/* The cudaStream_t the graph launches on (as void*). */
void *eprem_gpu_ensemble_stream(eprem_gpu_ensemble *ens);

/* ---- Learned surrogate building blocks (no reference counterpart) ---------
 * c[m x n] = a[m x k] * bt[n x k]^T (+ bias[n]) on the tensor cores
 * (tcgen05, bf16 operands, fp32 accumulation in tensor memory).  Device
 * pointers: a, bt bf16 with k contiguous (lda, ldb >= k, multiples of 8), c
 * fp32 (ldc >= n), bias fp32 or NULL; k a multiple of 8.  Runs on `stream`
 * (a cudaStream_t, NULL for the default stream) and synchronizes it.
 * EPREM_GPU_ERR_CUDA if a wait on the tensor cores timed out. */
int eprem_gpu_gemm_bf16(const void *a, int lda, const void *bt, int ldb, const float *bias,
                        float *c, int ldc, int m, int n, int k, void *stream);

/* ---- Split form and the learned surrogate (no reference counterpart) -------
 * Node phase of each EP sub-step:
 *   REFERENCE  the reference's scheme: relaxation inside every streaming
 *              sub-cycle, then focusing and adiabatic change;
 *   SPLIT      streaming without relaxation; per (node, energy) row the
 *              focusing sub-cycles and then one exact relaxation over the
 *              sub-step, f = iso + (f - iso) exp(-dt/tau); adiabatic change;
 *   SURROGATE  as SPLIT, with the row step predicted by the surrogate MLP,
 *              projected to conserve sum_mu f exactly (FP64 sums), and
 *              recomputed by the SPLIT kernel wherever its Crank-Nicolson
 *              residual exceeds the surrogate's tolerance;
 *   SURROGATE_FOCUS  the reference's scheme (relaxation inside streaming)
 *              with the focusing sub-cycles predicted by the surrogate,
 *              projected and checked the same way (fallback: the focusing
 *              kernel).  The operator splitting is the reference's.
 * All but REFERENCE need the FP32 form with Euler operators, focusing on and
 * 40 mu cells.  SPLIT and SURROGATE change the reference's operator
 * splitting; every form's flux error against the FP64 reference form is
 * measured and reported. */
enum {
  EPREM_NODE_PHASE_REFERENCE = 0,
  EPREM_NODE_PHASE_SPLIT = 1,
  EPREM_NODE_PHASE_SURROGATE = 2,
  EPREM_NODE_PHASE_SURROGATE_FOCUS = 3
};
typedef struct eprem_gpu_surrogate eprem_gpu_surrogate;

/* MLP 48 -> 256 -> 256 -> 48 (tanh-form GELU), bf16 weights and fp32
 * accumulation on the tensor cores; fp32 master parameters, Adam.  Inputs:
 * ln f(mu) minus its mean (40), asinh(a dt/dmu), asinh(b dt/dmu), 1 -
 * exp(-dt/tau), zero padding; outputs: the change of ln f(mu) (40 used).
 * chunk_rows: rows per inference chunk (device buffers ~2.3 KB per row;
 * 0 = 524288).  Weights start Xavier-uniform from splitmix64(seed). */
int eprem_gpu_surrogate_create(uint64_t seed, int chunk_rows, eprem_gpu_surrogate **out);
int eprem_gpu_surrogate_destroy(eprem_gpu_surrogate *s);
/* Parameters, fp32, flat: W1[256][48], b1[256], W2[256][256], b2[256],
 * W3[48][256], b3[48] (weights as [out][in]). */
int64_t eprem_gpu_surrogate_num_params(void);
int eprem_gpu_surrogate_get_params(eprem_gpu_surrogate *s, float *params, int64_t n);
int eprem_gpu_surrogate_set_params(eprem_gpu_surrogate *s, const float *params, int64_t n);
/* Training set: room for `capacity` rows (emptied); collect adds the rows of
 * the run's current state chosen at `rate` by a hash of (seed, row), each
 * with the run's plain row step as the target (the focusing alone for a run
 * in the reference scheme, focusing + relaxation for a split-form run);
 * *total = rows held. */
int eprem_gpu_surrogate_reserve(eprem_gpu_surrogate *s, int64_t capacity);
int eprem_gpu_surrogate_collect(eprem_gpu_surrogate *s, eprem_gpu_run *run, double rate,
                                uint64_t seed, int64_t *total);
/* `steps` Adam steps (learning rate lr) on random windows of `batch` rows
 * (a multiple of 8, <= 16384) by the library's forward and backward
 * kernels; *last_loss = mean squared error of the last batch. */
int eprem_gpu_surrogate_train(eprem_gpu_surrogate *s, int steps, int batch, double lr,
                              double *last_loss);
/* One forward and backward pass on host rows (x: rows x 48, t: rows x 40,
 * rows a multiple of 8, <= 16384): mean squared error and its gradient in
 * the parameter layout above; no update.  evaluate: outputs y (rows x 48). */
int eprem_gpu_surrogate_loss_grad(eprem_gpu_surrogate *s, const float *x, const float *t,
                                  int rows, double *loss, float *grad);
int eprem_gpu_surrogate_evaluate(eprem_gpu_surrogate *s, const float *x, int rows, float *y);
/* Residual tolerance: the `quantile` of the collected plain rows' residuals
 * times `margin`; or set directly. */
int eprem_gpu_surrogate_calibrate(eprem_gpu_surrogate *s, double quantile, double margin,
                                  double *tol);
int eprem_gpu_surrogate_set_tolerance(eprem_gpu_surrogate *s, double tol);
/* Tolerance from the true error instead: the network runs on up to `rows`
 * collected rows (0: all), whose plain step is known; the tolerance becomes
 * the largest residual below which every one of them is within `target` of
 * its plain step (max over mu of |f_net - f_plain| over the row's mean).
 * *kept: fraction of those rows the check then keeps; *within: fraction
 * within target at all (what a check with the plain step itself would keep). */
int eprem_gpu_surrogate_calibrate_error(eprem_gpu_surrogate *s, double target, int64_t rows,
                                        double *tol, double *kept, double *within);
/* Choose the node phase of a run (the surrogate for SURROGATE, else NULL). */
int eprem_gpu_set_node_phase(eprem_gpu_run *run, int mode, eprem_gpu_surrogate *s);
/* Rows the surrogate kept and rows recomputed by the plain kernel since the
 * node phase was set. */
int eprem_gpu_surrogate_counts(eprem_gpu_run *run, uint64_t *kept, uint64_t *fallback);

/* Message of the last failure on this thread ("" if none). */
const char *eprem_gpu_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* EPREM_GPU_H */
