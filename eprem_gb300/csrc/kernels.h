// kernels.h -- host-side launch entry points of the kernels (one per .cu).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"

namespace eprem {

// geometry.cu
int launch_geometry(const RunView &r, cudaStream_t st, double norm_radius, double neg_beta,
                    int mfp_type, double mfp_power, double bs_au, uint64_t *launches);
int setup_geometry_attrs(int N);

// stream.cu -- DiffuseStreamData (+ seedPopulationCheck)
struct StreamPlan {
  int mmax;      // register slots per thread (>= M)
  int threads;   // threads per CTA
  int cluster;   // CTAs per (stream, energy) slab
  int reg_coef;  // coefficients in registers (1), shared memory (0); 2: stream2.cu
  int packed;    // stream2.cu: fp32x2 arithmetic on pairs of mu cells
  int filled;    // stream2.cu: M fills the bin, m0 = M/2 (guards known at compile time)
  int npt;       // stream2.cu: list nodes per thread
  int mirror;    // stream2.cu: mu < 0 half in mirror order, one coefficient per two cells
                 // (1 formed on the sub-cycle loop, 2 from shared memory)
};
// bc: the run has the seed boundary (the mirrored kinds need it)
int plan_stream(int precision, int N, int M, int m0, int variant, bool bc, StreamPlan *plan);
int launch_stream(const RunView &r, const StreamPlan &plan, int m0, cudaStream_t st,
                  uint64_t *launches);
int launch_seed_check(const RunView &r, cudaStream_t st, uint64_t *launches);
// stream2.cu -- FP32 streaming, two list nodes per thread (plan.reg_coef == 2)
// shape: 0 automatic, k >= 1 the k-th CTA shape of M's bin (stream2_shape_count)
// mirror: 0, or the mirrored kind (1, 2: StreamPlan::mirror), which needs filled and bc
int plan_stream2(int N, int M, int m0, bool packed, bool filled, int mirror, bool bc, int shape,
                 StreamPlan *plan);
int stream2_shape_count(int M);
// The packed kinds over the slabs of several runs of one plan: the runs'
// views (a kernel parameter) and items[i] = (run index, stream, energy, 0)
constexpr int kMultiRuns = 64;
struct MultiRunViews {
  RunView v[kMultiRuns];
  int m0[kMultiRuns];
};
int launch_stream2_multi(const StreamPlan &pl, const MultiRunViews &mv, const int4 *items,
                         int n_items, cudaStream_t st, uint64_t *launches);
// once per updateEnergeticParticles call, before the stream2 launches
int launch_stream2_coef(const RunView &r, cudaStream_t st, uint64_t *launches);
int launch_stream2(const RunView &r, const StreamPlan &plan, int m0, cudaStream_t st,
                   uint64_t *launches);
// seedPopulationCheck alone in the FP32 form (rows renormalised)
int launch_seed_check32(const RunView &r, cudaStream_t st, uint64_t *launches);

// node.cu -- AdiabaticFocusing + AdiabaticChange
struct NodePlan {
  int pmax;        // register slots per thread (>= max(E, M); FP32 form: >= M)
  int pcol;        // FP32 form: register slots of a change column (>= E)
  int threads;     // threads per CTA
  int nodes;       // nodes per CTA
  size_t smem;     // dynamic shared memory bytes
  int fast32;      // FP32 form with Euler operators: node32.cu
};
int plan_node(int precision, int E, int M, NodePlan *plan);
int launch_node(const RunView &r, const NodePlan &plan, cudaStream_t st, uint64_t *launches);
// node32.cu -- FP32-form focusing + change (Euler operators)
int plan_node32(int E, int M, NodePlan *plan);
int launch_node32(const RunView &r, const NodePlan &plan, cudaStream_t st, uint64_t *launches);
// once per updateEnergeticParticles call, before the first launch_node32
int launch_node32_setup(const RunView &r, cudaStream_t st, uint64_t *launches);
// The node phase (focusing then change, both on) of several runs of one mu
// count and one plan in two launches; a run's own launches are the same
// kernels over one view.  foff / coff: each run's first focusing / change
// CTA (prefix sums of node32_blocks), n runs.
struct NodeRunViews {
  RunView v[kMultiRuns];
  int foff[kMultiRuns + 1], coff[kMultiRuns + 1];
  int n;
};
void node32_blocks(const RunView &r, int *focus_blocks, int *change_blocks);
int launch_node32_multi(const NodePlan &pl, const NodeRunViews &nv, cudaStream_t st,
                        uint64_t *launches);

// mhd.cu -- updateMhd (analytic), moveNodes, omnidirectional flux, f conversion
struct MhdParams {
  double r_scale, t_del, mhd_us, mhd_ns_au, mhd_bs_au, omega_sun;
  int ideal_shock;
  double sharp, scale_len, jump, falloff, speed, init_time, theta, phi, width;
};
// tg_dev: the run's time on the device (t = *tg_dev + t_global), or null
int launch_update_mhd(const RunView &r, const MhdParams &p, double t_global, cudaStream_t st,
                      uint64_t *launches, const double *tg_dev = nullptr);
int launch_advance_time(double *t_dev, double dt, cudaStream_t st, uint64_t *launches);
int launch_seed_population(const RunView &r, unsigned long long seed, double perturb,
                           cudaStream_t st, uint64_t *launches);
int launch_move_nodes(const RunView &r, double dt, cudaStream_t st, uint64_t *launches);
int launch_omni_flux(const RunView &r, double *out, cudaStream_t st, uint64_t *launches);
int launch_ripple_f(const RunView &r, const double *tmpl, cudaStream_t st, uint64_t *launches);

// shell.cu -- cross-field (shell) diffusion (DiffuseShellData, ShellData)
int launch_shell_coef(const RunView &r, const int *news, double kperxkpar, void *del,
                      cudaStream_t st, uint64_t *launches);
// xout: the FP32 form's output row exponents (null in FP64); drift: the
// gather of DriftShellData (lists and fractions of launch_drift_coef)
int launch_shell_diffuse(const RunView &r, const int *ent, int L, const void *del, void *out,
                         short *xout, cudaStream_t st, uint64_t *launches, bool drift = false);
// DriftShellData's fractions, Real[N][E][S][4], from r.curl and the positions
int launch_drift_coef(const RunView &r, const int *news, void *del, cudaStream_t st,
                      uint64_t *launches);
// FP32 form: rows [row0, row0 + nrows) of view r between an FP64 staging
// buffer and the device's rows with their exponents
int launch_convert_f(const RunView &r, size_t row0, size_t nrows, double *stage, int to_device,
                     cudaStream_t st, uint64_t *launches);

// mas.cu -- MAS background (updateMhd MHD_MAS branch, masMoveNodes)
struct MasSlotDev {
  const float *data[EPREM_MAS_NFIELDS];
  const float *mesh[EPREM_MAS_NFIELDS][3];
  int dims[EPREM_MAS_NFIELDS][3];
};
struct MasView {
  MasSlotDev s0, s1;
  double s_cor, phi_offset, radial_max, v_min, r_scale, omega_sun;
  int cor_rotate_fake, rotate_solution;
};
int launch_mas_update_mhd(const RunView &r, const MasView &mv, double t_del, cudaStream_t st,
                          uint64_t *launches);
int launch_mas_move_nodes(const RunView &r, const MasView &mv, double dt, cudaStream_t st,
                          uint64_t *launches);

// mlp.cu -- tcgen05 BF16 GEMM C = A * Bt^T (+ bias) of the learned surrogate;
// err: device int set to 1 when a wait on the tensor cores timed out
int launch_gemm_bf16(const void *A, int lda, const void *Bt, int ldb, const float *bias,
                     float *C, int ldc, int M, int N, int K, int *err, cudaStream_t st);

// surrogate.cu -- split focusing + relaxation step and the learned surrogate
// (40 mu cells, FP32 form); row ranges [row0, row0 + nrows) of the S*N*E rows
int launch_split_focus_relax(const RunView &r, size_t row0, size_t nrows, const uint8_t *mask,
                             cudaStream_t st, uint64_t *launches);
int launch_surr_sample(const RunView &r, float *xs, float *ts, unsigned long long *count,
                       unsigned long long cap, unsigned long long seed, float rate,
                       cudaStream_t st);
int launch_surr_features(const RunView &r, size_t row0, size_t nrows, void *X, cudaStream_t st,
                         uint64_t *launches);
int launch_surr_apply(const RunView &r, size_t row0, size_t nrows, const float *Y, int ldy,
                      float tol, uint8_t *reject, unsigned long long *counts, cudaStream_t st,
                      uint64_t *launches);
int launch_surr_residual(const float *xs, const float *ts, size_t n, const float *mu32,
                         float *res, cudaStream_t st);
int launch_surr_calib(const float *xs, const float *ts, const float *Y, int ldy, size_t n,
                      const float *mu32, float *res, float *err, cudaStream_t st);
int launch_to_bf16(const float *in, void *out, size_t n, cudaStream_t st);
int launch_gelu_bf16(const float *Z, void *H, size_t n, cudaStream_t st);
int launch_mse_grad(const float *Y, const float *T, size_t rows, float *dY, void *dYb,
                    double *loss, cudaStream_t st);
int launch_gelu_back(const float *dH, const float *Z, float *dZ, void *dZb, size_t n,
                     cudaStream_t st);
int launch_transpose_bf16(const void *in, void *out, int R, int C, cudaStream_t st);
int launch_colsum(const float *in, int R, int C, float *out, cudaStream_t st);
int launch_adam(float *p, const float *g, float *m, float *v, size_t n, float lr, int step,
                cudaStream_t st);

}  // namespace eprem
