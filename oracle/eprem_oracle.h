/*
 * eprem_oracle.h -- CPU restatement of EPREM's per-timestep energetic-particle
 * update, used ONLY as the checker in tests/, in __graft_entry__.smoke() and
 * as bench.py's CPU baseline.  It is test infrastructure: no product code path
 * calls it, links it or falls back to it.
 *
 * It follows the reference C operation by operation (each function cites the
 * reference file:line it restates) so that, compiled with
 * -ffp-contract=off, it reproduces the reference bit for bit.  That claim is
 * checked in tests/test_oracle_vs_reference.py against the reference's own
 * functions compiled from source (oracle/Makefile -> oracle/_ref/).
 *
 * Data layout and parameter structs are those of include/eprem_gpu.h.
 */
#ifndef EPREM_ORACLE_H
#define EPREM_ORACLE_H

#include "../include/eprem_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* initEnergeticParticlesGrids (src/energeticParticlesInit.c:36-100):
 * fills egrid/vgrid/vgrid_i/pgrid [E], rigidity [E], mugrid [M]; returns
 * dlnp and dmu through the pointers. */
void orc_build_grids(int num_energies, int num_mu, double e_min_mev,
                     double e_max_mev, double mass, double charge,
                     double rigidity_power, double *egrid, double *vgrid,
                     double *vgrid_i, double *pgrid, double *rigidity,
                     double *mugrid, double *dlnp, double *dmu);

/* sepSeedFunction (src/energeticParticlesBoundary.c:67-116). */
double orc_seed_function(const eprem_params_t *p, double energy, double r);

/* setRuntimeConstants-style defaults of the reference getParams
 * (src/configuration.c:58-217, 325-348) for the members of eprem_params_t. */
void orc_default_params(eprem_params_t *p);

/* updateEnergeticParticles (src/energeticParticles.c:70-203) over all streams.
 * f: S*N*E*M, nodes: EPREM_NODE_NFIELDS*S*N (fields RX..DUPAR read; DS,
 * BMAG_PLUS, BMAG_MINUS written).  stats accumulate (max / min) into *stats,
 * which the caller initialises.  nthreads > 1 splits the streams across
 * POSIX threads (the streams are independent when drift and shell diffusion
 * are off, which this path requires).  Returns EPREM_GPU_OK or a status; the
 * failing location is written to errbuf (if non-NULL, 256 bytes). */
int orc_update_energetic_particles(const eprem_dims_t *d, const eprem_params_t *p,
                                   const eprem_grids_t *g, double *f, double *nodes,
                                   eprem_ep_stats_t *stats, int nthreads,
                                   char *errbuf);

/* Same, restricted to streams [s0, s1) -- the unit the CPU baseline times. */
int orc_update_energetic_particles_range(const eprem_dims_t *d,
                                         const eprem_params_t *p,
                                         const eprem_grids_t *g, double *f,
                                         double *nodes, int s0, int s1,
                                         eprem_ep_stats_t *stats, int nthreads,
                                         char *errbuf);

/* updateEnergeticParticles with useShellDiffusion on: after each sub-step's
 * streaming, focusing and change of all streams, DiffuseShellData
 * (src/energeticParticles.c:419-554) couples the streams of every shell,
 * with the perpendicular neighbour lengths of ShellData (:254-413) formed
 * from the node positions and B at the start of the call, as the driver
 * calls ShellData right before updateEnergeticParticles (src/eprem.c:647-671).
 * news: S*4 stream indices (face*R*C + row*C + col) of each stream's north,
 * east, west and south neighbour -- the Node_t links n, e, w, s
 * (src/cubeShellStruct.h), the same on every shell.  kperxkpar:
 * config.kperxkpar. */
int orc_update_energetic_particles_news(const eprem_dims_t *d, const eprem_params_t *p,
                                        const eprem_grids_t *g, double *f, double *nodes,
                                        const int32_t *news, double kperxkpar,
                                        eprem_ep_stats_t *stats, int nthreads,
                                        char *errbuf);

/* updateMhd for the analytic background (src/flow.c:36-154). */
int orc_update_mhd(const eprem_dims_t *d, const eprem_params_t *p,
                   double *nodes, double t_global);
/* The same with useDrift on: also curl(B)/B^2 of every node (mhdCurlBoverB2
 * with curlBoverB2, src/flow.c:127-128, :479-616), curl[3][S*N] (r, theta,
 * phi components). */
int orc_update_mhd_curl(const eprem_dims_t *d, const eprem_params_t *p,
                        double *nodes, double t_global, double *curl);
/* updateEnergeticParticles with the perpendicular steps after each
 * sub-step: DiffuseShellData when shell_on, then DriftShellData
 * (src/energeticParticles.c:561-801) when drift is non-NULL, with the
 * curl(B)/B^2 of orc_update_mhd_curl. */
int orc_update_energetic_particles_perp(const eprem_dims_t *d, const eprem_params_t *p,
                                        const eprem_grids_t *g, double *f, double *nodes,
                                        const int32_t *news, int shell_on, double kperxkpar,
                                        const eprem_drift_params_t *drift, const double *curl,
                                        eprem_ep_stats_t *stats, int nthreads, char *errbuf);

/* moveNodes (src/simCore.c:737-785) with delrFlow (src/flow.c:162-196). */
int orc_move_nodes(const eprem_dims_t *d, const eprem_params_t *p,
                   double *nodes, double dt);

/* 2 E mean_mu f per (stream,node,E) (src/unifiedOutput.c:153-180 without the
 * unit scale). out: S*N*E. */
void orc_omni_flux(const eprem_dims_t *d, const eprem_grids_t *g,
                   const double *f, double *out);

/* MAS background: two time slots, the time factor s_cor and the phi offset,
 * as the reference's readMAS globals hold them. */
typedef struct {
  const eprem_mas_slice_t *slot0, *slot1;
  double s_cor, phi_offset;
  eprem_mas_params_t p;
} orc_mas_t;

/* updateMhd with mhdGridStatus == MHD_MAS (src/flow.c:36-154 with
 * masGetNode src/masInterp.c:31-68). */
int orc_mas_update_mhd(const eprem_dims_t *d, const eprem_params_t *p, double *nodes,
                       const orc_mas_t *mas, double t_global);
/* masMoveNodes (src/masInterp.c:1344-1393). */
int orc_mas_move_nodes(const eprem_dims_t *d, const eprem_params_t *p, double *nodes,
                       const orc_mas_t *mas, double dt);
#ifdef __cplusplus
}
#endif
#endif
