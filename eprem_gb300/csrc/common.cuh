// common.cuh -- device-side state and helpers shared by the EPREM kernels.
//
// One run = one set of streams held entirely in this GPU's HBM:
//   f      [S][N][E][M] (Real = double for the plain form, float for the FP32
//          form), mu fastest: the reference eParts order (src/global.h:61)
//          without its ghost shell.
//   nodes  [NF][S*N] doubles, one row per Node_t member used by the hot path.
// plus per-call scratch (stream lists, per-node seed/mean-free-path factors)
// and a small status/statistics block.
#pragma once

#include <cfloat>
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/eprem_gpu.h"

namespace eprem {

constexpr double kPi = 3.1415926535897932;
constexpr double kMp = 1.6726e-24;
constexpr double kMev = 1.6022e-6;
constexpr double kC = 2.99792458e10;
constexpr double kAu = 1.495978707e13;
constexpr double kVerySmall = 1.0e-33;
constexpr double kTau = kAu / kC;
constexpr double kDay = kTau / (24.0 * 60.0 * 60.0);
constexpr double kMhdDensityNorm = 1.0;

// Device status: first failure wins.
struct DevStatus {
  int code;      // EPREM_GPU_ERR_* or 0
  int where;     // 1 stream, 2 focusing, 3 change, 4 geometry, 5 seed check
  int stream, node, energy, mu;
  int max_change, max_focus, max_stream;
  unsigned long long min_tau_bits;        // min over positive doubles
  unsigned long long stream_cs, focus_cs, change_cs;  // cells x sub-cycles per operator
};

// Per-energy constants computed on the host at create time with the host libm
// (the reference evaluates them with the C library too).
struct EnergyConsts {
  double egrid, vgrid, vgrid_i;
  double rig_lamo;       // rigidity[E] * lamo              (src/meanFreePath.c:15)
  double seed_power;     // pow(E/normE1, -gamma)           (src/energeticParticlesBoundary.c:101)
  double seed_exp;       // exp(-(E/normE0))                (:102)
  float v32, vi32;       // vgrid, vgrid_i rounded to float (FP32 stencils)
};

// Per-node coefficients of the FP32 focusing / change kernels, fixed for one
// updateEnergeticParticles call (a node's MHD fields, ds and |B+-| do not
// change during it).  ok = 0 for the spawn node, which is not updated.
struct NodeCoef32 {
  int ok, ns_f, ns_c, pad0;
  float dlnbds, dupar, b, scale_f;  // focusing: a_E = -v dlnbds - (2/v) dupar
  float cool, dlnb, dlnn, scale_c;  // change (rates per unit time)
  float bc0, bc1, pad1, pad2;       // ln seed at the first and last energy
};

struct RunView {
  int S, N, E, M;
  int precision;
  void *f;                 // Real*
  double *nodes;           // [NF][S*N]
  const double *mugrid;    // [M]
  const EnergyConsts *ec;  // [E]
  const float *mugrid32;   // [M]     mugrid rounded to float
  // per-call scratch
  int *list;               // [S][N]  stream list (GetStreamList shellList)
  int *list_size;          // [S]
  double *ds_i;            // [S][N]  1/ds of list segments (FindSegmentLengths)
  double *ds_min;          // [S]
  double *seed_radial;     // [S*N]   pow(r/normRadius, -beta)
  double *mfp_node;        // [S*N]   pow(r*rScale, a) or pow(BsAu/B, b)
  NodeCoef32 *coef32;      // [S*N]   FP32 form only
  float4 *scoef;           // [S][E][N] FP32 streaming coefficients (stream2.cu)
  DevStatus *status;
  // parameters
  double r_scale, dt, dt_full, dmu, dlnp;
  double norm_j0, bf_xi, dsh_min, damp_cooling;
  double f_scale, f_unscale;  // device f = f * f_scale (2^kF32Shift in the FP32 form, else 1)
  double ln_f_shift;          // ln f_scale (0 in FP64): the change operator works on ln f itself
  // A view of streams [s_base, s_base + S) of the run (stream_range_view):
  // node field k of node g is nodes[k * node_stride + g]
  size_t node_stride;
  int s_base;
  int num_ep_steps, max_subcycles;
  int check_seed, use_bc, use_stream, use_focus, use_change;
  int focus_alg, change_alg;
  int relax_in_stream;     // 0 in the split form (relaxation with the focusing, node phase)
};

__device__ __forceinline__ double *node_field(const RunView &r, int field) {
  return r.nodes + (size_t)field * r.node_stride;
}

__device__ __forceinline__ void set_error(DevStatus *st, int code, int where, int s, int k, int e,
                                          int m) {
  if (atomicCAS(&st->code, 0, code) == 0) {
    st->where = where;
    st->stream = s;
    st->node = k;
    st->energy = e;
    st->mu = m;
  }
}

// The same, for a stream index s of the view r (reported as the run's stream).
__device__ __forceinline__ void set_error(const RunView &r, int code, int where, int s, int k,
                                          int e, int m) {
  set_error(r.status, code, where, s < 0 ? s : s + r.s_base, k, e, m);
}

// Non-negative doubles order like their bit patterns.
__device__ __forceinline__ void atomic_min_pos(unsigned long long *addr, double v) {
  atomicMin(addr, (unsigned long long)__double_as_longlong(v));
}
__device__ __forceinline__ void atomic_max_pos(unsigned long long *addr, double v) {
  atomicMax(addr, (unsigned long long)__double_as_longlong(v));
}

// The FP32 form holds f multiplied by 2^kF32Shift.  Streaming,
// isotropisation and focusing are linear in f, so the shift changes none of
// their results beyond rounding.  Adiabatic change advects ln f in flux form
// with a velocity that varies along ln p, which is not invariant under
// ln f -> ln f + const: its kernels take ln f_scale off on load (and off the
// seed boundary values) and put it back before the exponential.  The shift
// moves the float window from [1.2e-38, 3.4e38]
// to [6.4e-58, 1.8e19] in EPREM's normalised units, where the distributions
// of real runs live: their far tails (f down to 1e-240 in the MAS testsuite
// runs) then floor 20 decades lower, so floored cells stop feeding the
// fluxes within 30 decades of the peak.  Conversions, seeds and the flux
// apply the shift; FP64 runs use a scale of 1.
constexpr int kF32Shift = 64;

// sepSeedFunction (src/energeticParticlesBoundary.c:67-116) with the
// node-only factor (radial term) and the energy-only factors precomputed:
// normJHe = normJ0 * radial * power * exp, then /xi, /(2E), floor DBL_MIN.
__device__ __forceinline__ double seed_value(const RunView &r, const EnergyConsts &ec,
                                             double radial) {
  double normJHe = r.norm_j0 * radial * ec.seed_power * ec.seed_exp;
  double normJ = normJHe / r.bf_xi;
  double normf = normJ / (2.0 * ec.egrid);
  if (normf < DBL_MIN) normf = DBL_MIN;
  return normf * r.f_scale;  // in the device's units of f (exact: a power of two)
}

// Floor value below which the reference resets f (DBL_MIN); the FP32 form
// uses the smallest normal float instead.
template <typename Real> struct Floor;
template <> struct Floor<double> { static __device__ __forceinline__ double v() { return DBL_MIN; } };
template <> struct Floor<float> { static __device__ __forceinline__ float v() { return FLT_MIN; } };

template <typename Real> __device__ __forceinline__ Real to_real(double x);
template <> __device__ __forceinline__ double to_real<double>(double x) { return x; }
template <> __device__ __forceinline__ float to_real<float>(double x) {
  float v = (float)x;
  return v < FLT_MIN ? FLT_MIN : v;
}

template <typename Real> __device__ __forceinline__ Real log_r(Real x);
template <> __device__ __forceinline__ double log_r<double>(double x) { return log(x); }
template <> __device__ __forceinline__ float log_r<float>(float x) { return logf(x); }
template <typename Real> __device__ __forceinline__ Real exp_r(Real x);
template <> __device__ __forceinline__ double exp_r<double>(double x) { return exp(x); }
template <> __device__ __forceinline__ float exp_r<float>(float x) { return expf(x); }

template <typename Real> __device__ __forceinline__ bool bad_value(Real v, int *code) {
  if (isnan(v)) { *code = EPREM_GPU_ERR_NAN; return true; }
  if (isinf(v)) { *code = EPREM_GPU_ERR_INF; return true; }
  return false;
}

}  // namespace eprem
