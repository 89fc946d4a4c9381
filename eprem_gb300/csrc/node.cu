// node.cu -- adiabatic focusing and adiabatic change per node (K23).
//
// Restates, for every node but the innermost of each stream (innerComputeShell,
// src/mpiInit.c:105-109):
//   AdiabaticFocusing  (src/energeticParticles.c:1537-1803) -- advection in mu
//     along each energy row, sub-cycled to the node's CFL limit;
//   AdiabaticChange    (src/energeticParticles.c:808-1077) -- advection of
//     ln f in ln p along each mu column, sub-cycled likewise;
// with the Euler upwind operators (:1084-1176, :1809-1895) in registers and
// the RK3-TVD / WENO3 variants (:1182-1427, :1902-2144) on a generic path.
//
// A CTA loads G consecutive node slabs (E x M each, contiguous in f) into
// shared memory; focusing gives each thread one (node, energy) row, change
// one (node, mu) column.  The CFL maxima are shared-memory atomic maxima of
// non-negative doubles; they and the sub-cycle counts are computed without
// fused multiply-adds so they match the reference's integers exactly.
#include "common.cuh"
#include "kernels.h"

namespace eprem {

constexpr int kNodeThreads = 128;
constexpr int kMaxNodesPerCta = 16;

__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }

// ---- generic operators on one line (row or column) in local memory --------
// Focusing operators act on a mu row of n cells with n+1 faces; change
// operators on an energy column.  They follow the reference loops exactly.
template <typename Real>
__device__ void op_focus_upwind(Real *f1, const Real *f, const Real *va, int n, Real dmu_i) {
  // src/energeticParticles.c:1809-1895 on one energy row
  Real flux_prev = (Real)0;
  for (int m = 1; m < n; m++) {
    Real v = va[m];
    Real fl = v * (v >= (Real)0 ? f[m - 1] : f[m]);
    if (m >= 2) f1[m - 1] = (fl - flux_prev) * dmu_i;
    flux_prev = fl;
    if (m == 1) f1[0] = fl * dmu_i;
  }
  f1[n - 1] = -flux_prev * dmu_i;
}

template <typename Real>
__device__ Real weno_flux(Real LNm2, Real LNm1, Real LN0, Real LP_1, Real LP0, Real LPp1) {
  // src/energeticParticles.c:1315-1342 / :2035-2062
  const Real cc = (Real)0.5, cm = (Real)0.5;
  const Real tm = (Real)(1.0 / 3.0), tcp = (Real)(2.0 / 3.0), tp = (Real)(1.0 / 3.0),
             tmc = (Real)(2.0 / 3.0);
  const Real eps = (Real)(10.0 * sqrt(DBL_MIN));
  Real p0m = ((Real)1 + cm) * LNm1 - cm * LNm2;
  Real p1m = cm * LNm1 + cc * LN0;
  Real p0p = ((Real)1 + cc) * LP0 - cc * LPp1;
  Real p1p = cc * LP0 + cm * LP_1;
  Real t;
  t = cm * (LNm1 - LNm2); Real B0m = (Real)4 * (t * t);
  t = cc * (LN0 - LNm1); Real B1m = (Real)4 * (t * t);
  t = cc * (LPp1 - LP0); Real B0p = (Real)4 * (t * t);
  t = cm * (LP0 - LP_1); Real B1p = (Real)4 * (t * t);
  t = eps + B0m; Real w0m = tp / (t * t);
  t = eps + B1m; Real w1m = tmc / (t * t);
  t = eps + B0p; Real w0p = tm / (t * t);
  t = eps + B1p; Real w1p = tcp / (t * t);
  Real wm = w0m + w1m, wp = w0p + w1p;
  Real um = (w0m / wm) * p0m + (w1m / wm) * p1m;
  Real up = (w0p / wp) * p0p + (w1p / wp) * p1p;
  return up + um;
}

template <typename Real>
__device__ Real line_alpha(const Real *va, int lo, int hi) {
  Real a = (Real)0;
  for (int i = lo; i <= hi; i++) a = fmax(a, fabs(va[i]));
  return a;
}

// WENO3 line operator; `change` selects the adiabatic-change boundary
// treatment (Dirichlet seed on inflow) over the focusing wall.
template <typename Real>
__device__ void op_weno3(Real *f1, const Real *f, const Real *va, int n, Real d, bool change,
                         Real bc0, Real bc1, Real *LP, Real *LN, Real *flux) {
  for (int m = 0; m < n; m++) {
    int lo, hi;
    if (m == 0) { lo = 0; hi = 3; }
    else if (m == 1) { lo = 0; hi = 4; }
    else if (m == n - 2) { lo = n - 4; hi = n; }
    else if (m == n - 1) { lo = n - 3; hi = n; }
    else { lo = m - 2; hi = m + 3; }
    Real alpha = line_alpha(va, lo, hi);
    LP[m] = (Real)0.5 * f[m] * va[m + 1] - alpha;
    LN[m] = (Real)0.5 * f[m] * va[m] + alpha;
  }
  for (int m = 2; m < n - 1; m++)
    flux[m] = weno_flux(LN[m - 2], LN[m - 1], LN[m], LP[m - 1], LP[m], LP[m + 1]);
  {
    Real v = va[1];
    flux[1] = v * (v >= (Real)0 ? f[0] : f[1]);
    v = va[n - 1];
    flux[n - 1] = v * (v >= (Real)0 ? f[n - 2] : f[n - 1]);
  }
  for (int m = 1; m < n - 1; m++) f1[m] = (flux[m + 1] - flux[m]) / d;
  if (!change) {
    Real v = va[1];
    f1[0] = v * (v <= (Real)0 ? f[1] : f[0]) / d;
    v = va[n - 1];
    f1[n - 1] = v * (-(v >= (Real)0 ? f[n - 2] : f[n - 1])) / d;
  } else {
    Real v = va[1];
    f1[0] = (v <= (Real)0) ? v * (f[1] - f[0]) / d : v * (f[0] - bc0) / d;
    v = va[n - 1];
    f1[n - 1] = (v >= (Real)0) ? v * (f[n - 1] - f[n - 2]) / d : v * (bc1 - f[n - 1]) / d;
  }
}

template <typename Real>
__device__ void op_change_upwind(Real *f1, const Real *f, const Real *va, int n, Real dlnp_i,
                                 Real bc0, Real bc1) {
  // src/energeticParticles.c:1084-1176 on one mu column
  Real flux_prev = (Real)0;
  for (int e = 1; e < n; e++) {
    Real v = va[e];
    Real fl = v * (v >= (Real)0 ? f[e - 1] : f[e]);
    if (e >= 2) f1[e - 1] = (fl - flux_prev) * dlnp_i;
    flux_prev = fl;
  }
  Real v = va[1];
  f1[0] = (v <= (Real)0) ? v * (f[1] - f[0]) * dlnp_i : v * (f[0] - bc0) * dlnp_i;
  v = va[n - 1];
  f1[n - 1] = (v >= (Real)0) ? v * (f[n - 1] - f[n - 2]) * dlnp_i : v * (bc1 - f[n - 1]) * dlnp_i;
}

// RK3-TVD (alg 2 upwind, alg 3 WENO3) over one line held in local memory,
// src/energeticParticles.c:958-1015 and :1683-1740.
template <typename Real, int P>
__device__ void line_rk3(Real *f, const Real *va, int n, int nsub, Real dts, bool change, int alg,
                         Real dgrid, Real bc0, Real bc1) {
  Real s1[P], f1[P], LP[P], LN[P], flux[P + 1];
  const Real di = (Real)1 / dgrid;
  auto op = [&](Real *out, const Real *in) {
    if (alg == 3)
      op_weno3(out, in, va, n, dgrid, change, bc0, bc1, LP, LN, flux);
    else if (change)
      op_change_upwind(out, in, va, n, di, bc0, bc1);
    else
      op_focus_upwind(out, in, va, n, di);
  };
  for (int s = 0; s < nsub; s++) {
    op(f1, f);
    for (int i = 0; i < n; i++) s1[i] = f[i] - dts * f1[i];
    op(f1, s1);
    for (int i = 0; i < n; i++)
      s1[i] = (Real)(3.0 / 4.0) * f[i] + (Real)(1.0 / 4.0) * s1[i] - (Real)(1.0 / 4.0) * dts * f1[i];
    op(f1, s1);
    for (int i = 0; i < n; i++)
      f[i] = (Real)(1.0 / 3.0) * f[i] + (Real)(2.0 / 3.0) * s1[i] - (Real)(2.0 / 3.0) * dts * f1[i];
  }
}

// ---- the node kernel --------------------------------------------------------
template <typename Real, int P>
__global__ void __launch_bounds__(kNodeThreads) k_node(RunView r, int G) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int E = r.E, M = r.M, N = r.N;
  const int EM = E * M;
  const int F = (E * (M + 1) > (E + 1) * M) ? E * (M + 1) : (E + 1) * M;
  double *vf = reinterpret_cast<double *>(smraw);                // [G][F] face velocities
  Real *slab = reinterpret_cast<Real *>(vf + (size_t)G * F);     // [G][E*M]
  __shared__ unsigned long long vmax_bits[kMaxNodesPerCta];
  __shared__ double n_a[kMaxNodesPerCta], n_b[kMaxNodesPerCta], n_c[kMaxNodesPerCta],
      n_d[kMaxNodesPerCta];
  __shared__ double n_bc0[kMaxNodesPerCta], n_bc1[kMaxNodesPerCta], n_dts[kMaxNodesPerCta];
  __shared__ int n_sub[kMaxNodesPerCta], n_ok[kMaxNodesPerCta];
  const int tid = threadIdx.x;
  const size_t SN = (size_t)r.S * N;
  const size_t g0 = (size_t)blockIdx.x * G;
  const int Gv = (int)((SN - g0) < (size_t)G ? (SN - g0) : (size_t)G);
  Real *fg = reinterpret_cast<Real *>(r.f) + g0 * EM;

  for (int i = tid; i < Gv * EM; i += kNodeThreads) slab[i] = fg[i];
  if (tid < Gv) n_ok[tid] = ((g0 + tid) % N) != 0;  // node 0 is the spawn node
  __syncthreads();

  const double dt = r.dt, dt_full = r.dt_full;
  // ------------------------------------------------------------- focusing
  if (r.use_focus) {
    if (tid < Gv) {
      const size_t g = g0 + tid;
      const double dupar = node_field(r, EPREM_NODE_DUPAR)[g] / dt_full;
      const double b = sub(mul(2.0, node_field(r, EPREM_NODE_DLNN)[g] / dt_full),
                           mul(3.0, node_field(r, EPREM_NODE_DLNB)[g] / dt_full));
      const double bp = node_field(r, EPREM_NODE_BMAG_PLUS)[g];
      const double bm = node_field(r, EPREM_NODE_BMAG_MINUS)[g];
      double dlnbds;
      if (bp == 0.0 || bm == 0.0)
        dlnbds = 0.0;
      else
        dlnbds = (log(bp) - log(bm)) / add(mul(2.0, node_field(r, EPREM_NODE_DS)[g]), DBL_MIN);
      n_a[tid] = dupar;
      n_b[tid] = b;
      n_c[tid] = dlnbds;
      vmax_bits[tid] = 0ull;
    }
    __syncthreads();
    // face velocities: v_avg(mu+1) = (vel(mu+1) + vel(mu)) / 2,
    // vel = (1 - mu^2)/2 (a + mu b), a = -v dlnB/ds - (2/v) DuPar/dt
    for (int it = tid; it < Gv * E * (M - 1); it += kNodeThreads) {
      const int g = it / (E * (M - 1));
      const int rem = it % (E * (M - 1));
      const int e = rem / (M - 1), j = rem % (M - 1);
      const double v = r.ec[e].vgrid;
      const double a = sub(mul(-v, n_c[g]), mul(2.0 / v, n_a[g]));
      const double m0 = r.mugrid[j], m1 = r.mugrid[j + 1];
      const double vel0 = mul(mul(0.5, sub(1.0, mul(m0, m0))), add(a, mul(m0, n_b[g])));
      const double vel1 = mul(mul(0.5, sub(1.0, mul(m1, m1))), add(a, mul(m1, n_b[g])));
      const double va = mul(0.5, add(vel1, vel0));
      vf[(size_t)g * F + e * (M + 1) + j + 1] = va;
      // the reference's `if (fabs(va) > vel_abs_max)` passes over a NaN
      if (!isnan(va)) atomic_max_pos(&vmax_bits[g], fabs(va));
    }
    __syncthreads();
    for (int it = tid; it < Gv * E; it += kNodeThreads) {
      double *row = vf + (size_t)(it / E) * F + (it % E) * (M + 1);
      row[0] = row[1];
      row[M] = row[M - 1];
    }
    if (tid < Gv) {
      const double vmax = __longlong_as_double((long long)vmax_bits[tid]);
      const double dt_stable = mul(0.9, r.dmu) / vmax;
      const double nsub = ceil(dt / dt_stable);
      int ns = 0;
      if (!(nsub <= (double)r.max_subcycles)) {
        if (n_ok[tid]) {
          const size_t g = g0 + tid;
          set_error(r, EPREM_GPU_ERR_SUBCYCLES, 2, (int)(g / N), (int)(g % N), -1, -1);
        }
      } else {
        ns = (int)nsub;
      }
      if (!n_ok[tid]) ns = 0;
      n_sub[tid] = ns;
      n_dts[tid] = dt / ns;
      if (n_ok[tid]) {
        atomicMax(&r.status->max_focus, ns);
        atomicAdd(&r.status->focus_cs, (unsigned long long)ns * EM);
      }
    }
    __syncthreads();
    const int alg = r.focus_alg;
    if (alg == 1) {  // pre-scale the faces by dt_sub/dmu for the Euler sweep
      for (int it = tid; it < Gv * E * (M + 1); it += kNodeThreads) {
        const int g = it / (E * (M + 1));
        vf[(size_t)g * F + it % (E * (M + 1))] *= n_dts[g] / r.dmu;
      }
      __syncthreads();
    }
    // one energy row per thread
    const Real fl_min = Floor<Real>::v();
    for (int it = tid; it < Gv * E; it += kNodeThreads) {
      const int g = it / E, e = it % E;
      const int ns = n_sub[g];
      Real *row = slab + (size_t)g * EM + e * M;
      const double *vrow = vf + (size_t)g * F + e * (M + 1);
      if (ns > 0 && alg == 1) {
        // Euler upwind with the face velocity pre-scaled by dt_sub/dmu:
        // f(mu) -= q(mu+1) f_up(mu+1) - q(mu) f_up(mu), walls at both ends.
        Real fr[P];
#pragma unroll
        for (int m = 0; m < P; ++m)
          if (m < M) fr[m] = row[m];
        for (int s = 0; s < ns; ++s) {
          Real gprev = (Real)0;
#pragma unroll
          for (int m = 0; m < P; ++m) {
            if (m < M) {
              Real gnext = (Real)0;
              if (m + 1 < M) {
                const Real qq = (Real)vrow[m + 1];
                gnext = qq * (qq >= (Real)0 ? fr[m] : fr[m + 1]);
              }
              fr[m] = fr[m] - (gnext - gprev);
              gprev = gnext;
            }
          }
        }
#pragma unroll
        for (int m = 0; m < P; ++m)
          if (m < M) row[m] = fr[m];
      } else if (ns > 0) {
        Real fl[P], va[P + 1];
        for (int m = 0; m < M; ++m) fl[m] = row[m];
        for (int m = 0; m <= M; ++m) va[m] = (Real)vrow[m];
        line_rk3<Real, P>(fl, va, M, ns, (Real)n_dts[g], false, alg, (Real)r.dmu, (Real)0,
                          (Real)0);
        for (int m = 0; m < M; ++m) row[m] = fl[m];
      }
      if (n_ok[g]) {
        int code = 0;
        for (int m = 0; m < M; ++m) {
          Real v = row[m];
          if (bad_value(v, &code)) {
            const size_t gg = g0 + g;
            set_error(r, code, 2, (int)(gg / N), (int)(gg % N), e, m);
          }
          row[m] = v < fl_min ? fl_min : v;
        }
      }
    }
    __syncthreads();
  }
  // --------------------------------------------------------- adiabatic change
  if (r.use_change) {
    if (tid < Gv) {
      const size_t g = g0 + tid;
      const double dlnbdt = node_field(r, EPREM_NODE_DLNB)[g] / dt_full;
      const double dlnndt = node_field(r, EPREM_NODE_DLNN)[g] / dt_full;
      n_a[tid] = node_field(r, EPREM_NODE_DUPAR)[g] / dt_full;
      n_b[tid] = dlnbdt;
      n_c[tid] = dlnndt;
      n_d[tid] = (dlnndt < 0) ? 1.0 - r.damp_cooling : 1.0;
      const double radial = r.seed_radial[g];
      n_bc0[tid] = log(seed_value(r, r.ec[0], radial));
      n_bc1[tid] = log(seed_value(r, r.ec[E - 1], radial));
      vmax_bits[tid] = 0ull;
    }
    __syncthreads();
    // vel(e, mu) = cool (a vi(e) + b): a = -mu DuPar/dt,
    // b = mu^2 (DlnN - DlnB)/dt + (1 - mu^2)/2 DlnB/dt; faces along energy
    for (int it = tid; it < Gv * EM; it += kNodeThreads) {
      const int g = it / EM, rem = it % EM;
      const int e = rem / M, m = rem % M;
      const double mu = r.mugrid[m];
      const double a = mul(-mu, n_a[g]);
      const double b = add(mul(mul(mu, mu), sub(n_c[g], n_b[g])),
                           mul(mul(0.5, sub(1.0, mul(mu, mu))), n_b[g]));
      const double vel = mul(n_d[g], add(mul(a, r.ec[e].vgrid_i), b));
      if (!isnan(vel)) atomic_max_pos(&vmax_bits[g], fabs(vel));
      if (e >= 1) {
        const double velm = mul(n_d[g], add(mul(a, r.ec[e - 1].vgrid_i), b));
        vf[(size_t)g * F + e * M + m] = mul(0.5, add(vel, velm));
      }
    }
    __syncthreads();
    for (int it = tid; it < Gv * M; it += kNodeThreads) {
      double *base = vf + (size_t)(it / M) * F;
      const int m = it % M;
      base[m] = base[M + m];
      base[E * M + m] = base[(E - 1) * M + m];
    }
    if (tid < Gv) {
      const double vmax = __longlong_as_double((long long)vmax_bits[tid]);
      const double dt_stable = mul(0.9, r.dlnp) / vmax;
      const double nsub = ceil(dt / dt_stable);
      int ns = 0;
      if (!(nsub <= (double)r.max_subcycles)) {
        if (n_ok[tid]) {
          const size_t g = g0 + tid;
          set_error(r, EPREM_GPU_ERR_SUBCYCLES, 3, (int)(g / N), (int)(g % N), -1, -1);
        }
      } else {
        ns = (int)nsub;
      }
      if (!n_ok[tid]) ns = 0;
      n_sub[tid] = ns;
      n_dts[tid] = dt / ns;
      if (n_ok[tid]) {
        atomicMax(&r.status->max_change, ns);
        atomicAdd(&r.status->change_cs, (unsigned long long)ns * EM);
      }
    }
    __syncthreads();
    const int alg = r.change_alg;
    if (alg == 1) {  // pre-scale the faces by dt_sub/dlnp for the Euler sweep
      for (int it = tid; it < Gv * (E + 1) * M; it += kNodeThreads) {
        const int g = it / ((E + 1) * M);
        vf[(size_t)g * F + it % ((E + 1) * M)] *= n_dts[g] / r.dlnp;
      }
      __syncthreads();
    }
    const Real fl_min = Floor<Real>::v();
    for (int it = tid; it < Gv * M; it += kNodeThreads) {
      const int g = it / M, m = it % M;
      if (!n_ok[g]) continue;
      const int ns = n_sub[g];
      Real *col = slab + (size_t)g * EM + m;  // stride M
      const double *vcol = vf + (size_t)g * F + m;  // face e at vcol[e*M]
      const Real bc0 = (Real)n_bc0[g], bc1 = (Real)n_bc1[g];
      // FP32 form: ln f itself is ln(stored) - fexp ln 2 (the row's exponent)
      const short *xrow = (sizeof(Real) == 4) ? r.fexp + (g0 + g) * E : nullptr;
      Real fc[P];
#pragma unroll
      for (int e = 0; e < P; ++e)
        if (e < E)
          fc[e] = log_r<Real>(col[e * M]) -
                  (xrow ? (Real)xrow[e] * (Real)0.69314718055994530942 : (Real)0);
      if (ns > 0 && alg == 1) {
        // Euler upwind in ln p, faces pre-scaled by dt_sub/dlnp; the end cells
        // use the reference's one-sided forms with the seed on inflow.
        for (int s = 0; s < ns; ++s) {
          const Real q1 = (Real)vcol[M];
          Real gprev = q1 * (q1 >= (Real)0 ? fc[0] : fc[1]);
          const Real d0 = (q1 <= (Real)0) ? q1 * (fc[1] - fc[0]) : q1 * (fc[0] - bc0);
          Real fold_prev = fc[0];
          fc[0] = fc[0] - d0;
#pragma unroll
          for (int e = 1; e < P; ++e) {
            if (e < E - 1) {
              const Real qq = (Real)vcol[(size_t)(e + 1) * M];
              const Real gnext = qq * (qq >= (Real)0 ? fc[e] : fc[e + 1]);
              fold_prev = fc[e];
              fc[e] = fc[e] - (gnext - gprev);
              gprev = gnext;
            } else if (e == E - 1) {
              const Real qq = (Real)vcol[(size_t)(E - 1) * M];
              const Real dl = (qq >= (Real)0) ? qq * (fc[e] - fold_prev) : qq * (bc1 - fc[e]);
              fc[e] = fc[e] - dl;
            }
          }
        }
      } else if (ns > 0) {
        Real fl[P], va[P + 1];
        for (int e = 0; e < E; ++e) fl[e] = fc[e];
        for (int e = 0; e <= E; ++e) va[e] = (Real)vcol[(size_t)e * M];
        line_rk3<Real, P>(fl, va, E, ns, (Real)n_dts[g], true, alg, (Real)r.dlnp, bc0, bc1);
        for (int e = 0; e < E; ++e) fc[e] = fl[e];
      }
      if constexpr (sizeof(Real) == 4) {
        // ln f stays in the slab; the row pass below renormalises and exponentiates
#pragma unroll
        for (int e = 0; e < P; ++e)
          if (e < E) col[e * M] = fc[e];
      } else {
        int code = 0;
#pragma unroll
        for (int e = 0; e < P; ++e) {
          if (e < E) {
            Real v = exp_r<Real>(fc[e]);
            if (bad_value(v, &code)) {
              const size_t gg = g0 + g;
              set_error(r, code, 3, (int)(gg / N), (int)(gg % N), e, m);
            }
            col[e * M] = v < fl_min ? fl_min : v;
          }
        }
      }
    }
    __syncthreads();
    if constexpr (sizeof(Real) == 4) {
      // FP32 form: each changed row gets the exponent that brings its largest
      // value to [2^kRowTop, 2^(kRowTop+1))
      for (int it = tid; it < Gv * E; it += kNodeThreads) {
        const int g = it / E, e = it % E;
        if (!n_ok[g]) continue;
        Real *row = slab + (size_t)g * EM + e * M;
        Real mx = row[0];
        for (int m = 1; m < M; ++m) mx = fmaxf(mx, row[m]);
        const float l2 = fminf(fmaxf(floorf(mx * 1.4426950408889634f), -1.0e6f), 1.0e6f);
        const int xn = clamp_exp(kRowTop - (int)l2);
        const float add = (float)xn * 0.6931471805599453f;
        int code = 0;
        for (int m = 0; m < M; ++m) {
          const float v = expf(row[m] + add);
          if (bad_value(v, &code)) {
            const size_t gg = g0 + g;
            set_error(r, code, 3, (int)(gg / N), (int)(gg % N), e, m);
          }
          row[m] = v < fl_min ? fl_min : v;
        }
        r.fexp[(g0 + g) * E + e] = (short)xn;
      }
      __syncthreads();
    }
  }
  for (int i = tid; i < Gv * EM; i += kNodeThreads) fg[i] = slab[i];
}

static const int kNodeBins[] = {8, 16, 24, 32, 48, 64};

int plan_node(int precision, int E, int M, NodePlan *plan) {
  const int mx = E > M ? E : M;
  int p = 0;
  for (int b : kNodeBins)
    if (mx <= b) { p = b; break; }
  if (!p) return EPREM_GPU_ERR_ARG;
  plan->pmax = p;
  plan->threads = kNodeThreads;
  const int F = (E * (M + 1) > (E + 1) * M) ? E * (M + 1) : (E + 1) * M;
  const size_t per = (size_t)F * sizeof(double) +
                     (size_t)E * M * (precision == EPREM_FP64 ? sizeof(double) : sizeof(float));
  const size_t budget = 96 * 1024;
  int G = (int)(budget / per);
  if (G > kMaxNodesPerCta) G = kMaxNodesPerCta;
  // enough rows to keep the CTA's threads busy, when that fits
  if (G < 1) G = 1;
  plan->nodes = G;
  plan->smem = per * G;
  if (plan->smem > 200 * 1024) return EPREM_GPU_ERR_ARG;
  return 0;
}

template <typename Real, int P>
static cudaError_t launch_node_t(const RunView &r, const NodePlan &pl, cudaStream_t st) {
  auto kern = k_node<Real, P>;
  cudaError_t err =
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pl.smem);
  if (err != cudaSuccess) return err;
  const size_t SN = (size_t)r.S * r.N;
  const unsigned blocks = (unsigned)((SN + pl.nodes - 1) / pl.nodes);
  kern<<<blocks, kNodeThreads, pl.smem, st>>>(r, pl.nodes);
  return cudaGetLastError();
}

template <typename Real>
static cudaError_t dispatch_node(const RunView &r, const NodePlan &pl, cudaStream_t st) {
  switch (pl.pmax) {
    case 8: return launch_node_t<Real, 8>(r, pl, st);
    case 16: return launch_node_t<Real, 16>(r, pl, st);
    case 24: return launch_node_t<Real, 24>(r, pl, st);
    case 32: return launch_node_t<Real, 32>(r, pl, st);
    case 48: return launch_node_t<Real, 48>(r, pl, st);
    default: return launch_node_t<Real, 64>(r, pl, st);
  }
}

int launch_node(const RunView &r, const NodePlan &plan, cudaStream_t st, uint64_t *launches) {
  cudaError_t err = r.precision == EPREM_FP64 ? dispatch_node<double>(r, plan, st)
                                              : dispatch_node<float>(r, plan, st);
  *launches += 1;
  return err == cudaSuccess ? 0 : EPREM_GPU_ERR_CUDA;
}

}  // namespace eprem
