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
constexpr double kQ = 4.80320425e-10;  // proton charge (esu), src/baseTypes.h:61

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
  float dvi32;           // vgrid_i[e+1] - vgrid_i[e-1] (0 at the ends), from FP64
  int seed_k;            // FP32 streaming seeds are held as seed * 2^seed_k, so that
                         // the energy-only factor of sepSeedFunction is near 1
  double drift_factor;   // (1/om1) p v / 3 of driftVelocity (src/energeticParticles.c:
                         // 210-246), p = exp(lnpmin + E dlnp); 0 without drift
};

// Per-node coefficients of the FP32 focusing / change kernels, fixed for one
// updateEnergeticParticles call (a node's MHD fields, ds and |B+-| do not
// change during it).  ok = 0 for the spawn node, which is not updated.
struct NodeCoef32 {
  int ok, ns_f, ns_c, pad0;
  float dlnbds, dupar, b, scale_f;  // focusing: a_E = -v dlnbds - (2/v) dupar
  float cool, dlnb, dlnn, scale_c;  // change (rates per unit time)
  // ln seed at the first and last energy as kbc * ln 2 + bc: the integer
  // part of log2 seed apart, so the change kernel can form the boundary
  // value relative to a row's exponent without losing the fraction
  float bc0, bc1;
  int kbc0, kbc1;
};

struct RunView {
  int S, N, E, M;
  int precision;
  void *f;                 // Real*
  short *fexp;             // [S][N][E] FP32 form: row exponents, f = f_stored * 2^-fexp
  double *curl;            // [3][S*N] curl(B)/B^2 (r, theta, phi) with drift on, else null
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

// The FP32 form holds each (stream, node, energy) row of M cells as floats
// with its own binary exponent: f = stored * 2^-fexp[row].  The reference's
// distributions span 230 decades across energies (the exponential cut-off
// of the seed spectrum), far beyond a float's 76, and its adiabatic change
// works on ln f, so a cell floored by the float range would feed a wrong
// ln f into its neighbours in energy; with one exponent per row every row
// keeps its own 76 decades.  A normalised row has its largest value in
// [2^kRowTop, 2^(kRowTop+1)): streaming, linear in f, brings every row of a
// (stream, energy) slab to the slab's common exponent on load and renormalises
// the slab; focusing keeps the row's exponent (its values grow at most M-fold);
// the change, in ln f, renormalises each row it writes.  Exponents stay at or
// below kRowExpMax, where the float floor FLT_MIN is the reference's DBL_MIN:
// no row ever floors below the reference's floor.
constexpr int kRowTop = 95;
constexpr int kRowExpMax = 896;   // FLT_MIN * 2^-896 = 2^-1022 = DBL_MIN
constexpr int kRowExpMin = -1000;
constexpr int kNoExp = -(1 << 20);  // log2 of a zero

__device__ __forceinline__ int clamp_exp(int k) {
  return k > kRowExpMax ? kRowExpMax : (k < kRowExpMin ? kRowExpMin : k);
}
// 2^k as a float, k in [-126, 127]
__device__ __forceinline__ float pow2f(int k) { return __int_as_float((k + 127) << 23); }
// x * 2^k for any k (two exact power-of-two steps; results below the float
// range underflow as a product would)
__device__ __forceinline__ float ldexp_f(float x, int k) {
  const int k1 = k > 127 ? 127 : (k < -126 ? -126 : k);
  int k2 = k - k1;
  k2 = k2 > 127 ? 127 : (k2 < -126 ? -126 : k2);
  return (x * pow2f(k1)) * pow2f(k2);
}
// floor(log2 x) of a non-negative float from its bits; kNoExp for zero
__device__ __forceinline__ int ilogb_f(float x) {
  const int b = __float_as_int(x) & 0x7fffffff;
  const int ex = b >> 23;
  if (ex) return ex - 127;
  const int m = b & 0x7fffff;
  return m ? -149 + (31 - __clz(m)) : kNoExp;
}
// the exponent that brings a row whose largest true value has floor(log2) = lg
// to [2^kRowTop, 2^(kRowTop+1))
__device__ __forceinline__ int row_exp_for(int lg) {
  return lg == kNoExp ? 0 : clamp_exp(kRowTop - lg);
}

// sepSeedFunction (src/energeticParticlesBoundary.c:67-116) with the
// node-only factor (radial term) and the energy-only factors precomputed:
// normJHe = normJ0 * radial * power * exp, then /xi, /(2E), floor DBL_MIN.
__device__ __forceinline__ double seed_value(const RunView &r, const EnergyConsts &ec,
                                             double radial) {
  double normJHe = r.norm_j0 * radial * ec.seed_power * ec.seed_exp;
  double normJ = normJHe / r.bf_xi;
  double normf = normJ / (2.0 * ec.egrid);
  if (normf < DBL_MIN) normf = DBL_MIN;
  return normf;
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
