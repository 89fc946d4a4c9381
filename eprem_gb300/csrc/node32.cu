// node32.cu -- focusing and adiabatic change in the FP32 form (K23').
//
// Same operators as node.cu (AdiabaticFocusing src/energeticParticles.c:
// 1537-1803, AdiabaticChange :808-1077, Euler upwind operators :1084-1176,
// :1809-1895), arranged for the FP32 pipe in three kernels:
//   * k_node32_setup, once per updateEnergeticParticles call: one warp per
//     node takes the FP64 CFL maxima (the sub-cycle counts) and the node's
//     coefficients.  A node's MHD fields, ds and |B+-| do not change during the
//     call, so the reference's per-sub-step recomputation yields the same
//     numbers every sub-step.  The maxima are exact whatever the order, so the
//     lanes split the energies / mu cells and reduce with shuffles:
//       - focusing's face velocity 1/4 (1-mu^2)(a_E + mu b) summed over two
//         cells is linear in a_E, so its maximum over energies lies on the
//         rows of the smallest and largest a_E;
//       - the change velocity cool (a_mu/v + b_mu) is linear in 1/v, which is
//         monotonic in energy, so its maximum lies on the first and last
//         energy rows.
//     Those rows are evaluated with the reference's expressions, without
//     fused multiply-adds;
//   * k_focus32, every EP sub-step: one thread per (node, energy) row, its M
//     cells and the split face coefficients max(q,0), min(q,0) in registers
//     (the CTA's rows staged through shared memory with coalesced copies);
//   * k_change32, every EP sub-step: one thread per (node, mu) column, whole
//     nodes per CTA (a warp reads consecutive mu of one energy: coalesced),
//     ln f in shared memory, each row renormalised to its own exponent.
// Both take a block of run views (NodeRunViews) and find their run from its
// first CTA: a run's own launch is one view, a lock-step ensemble's launch
// all the runs of one mu count -- the same compiled code either way, so an
// ensemble member's results equal its own run's bit for bit.
// No block barriers on the sub-cycle paths.  Only the
// Euler upwind algorithm (alg 1) runs here; RK3 / WENO3 use node.cu.
#include "common.cuh"
#include "kernels.h"

namespace eprem {

constexpr int kSetupWarps = 8;
constexpr int kFocusThreads = 128;
constexpr int kChangeThreads = 128;

__device__ __forceinline__ double m_(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double a_(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double s_(double a, double b) { return __dsub_rn(a, b); }

__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

__device__ __forceinline__ double warp_min(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w < v ? w : v;
  }
  return v;
}

// Focusing cell velocity at mu (src/energeticParticles.c:1620-1627), no FMA.
__device__ __forceinline__ double focus_vel(double mu, double a, double b) {
  return m_(m_(0.5, s_(1.0, m_(mu, mu))), a_(a, m_(mu, b)));
}

__global__ void __launch_bounds__(kSetupWarps * 32) k_node32_setup(RunView r) {
  __shared__ int s_max_f, s_max_c;
  __shared__ unsigned long long s_cs_f, s_cs_c;
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  if (threadIdx.x == 0) {
    s_max_f = s_max_c = 0;
    s_cs_f = s_cs_c = 0ull;
  }
  __syncthreads();
  const int E = r.E, M = r.M, N = r.N;
  const size_t SN = (size_t)r.S * N;
  const size_t g = (size_t)blockIdx.x * kSetupWarps + wib;
  if (g < SN) {
    const double dt = r.dt, dt_full = r.dt_full;
    const bool ok = (g % N) != 0;  // node 0 is the spawn node (innerComputeShell)
    const double dupar = node_field(r, EPREM_NODE_DUPAR)[g] / dt_full;
    const double dlnb = node_field(r, EPREM_NODE_DLNB)[g] / dt_full;
    const double dlnn = node_field(r, EPREM_NODE_DLNN)[g] / dt_full;
    NodeCoef32 c{};
    c.ok = ok;
    int ns_f = 0, ns_c = 0;
    if (r.use_focus) {
      const double b = s_(m_(2.0, dlnn), m_(3.0, dlnb));
      const double bp = node_field(r, EPREM_NODE_BMAG_PLUS)[g];
      const double bm = node_field(r, EPREM_NODE_BMAG_MINUS)[g];
      const double dlnbds =
          (bp == 0.0 || bm == 0.0)
              ? 0.0
              : (log(bp) - log(bm)) / a_(m_(2.0, node_field(r, EPREM_NODE_DS)[g]), DBL_MIN);
      double amin = DBL_MAX, amax = -DBL_MAX;
      for (int e = lane; e < E; e += 32) {
        const double v = r.ec[e].vgrid;
        const double a = s_(m_(-v, dlnbds), m_(2.0 / v, dupar));
        amin = a < amin ? a : amin;
        amax = a > amax ? a : amax;
      }
      amin = warp_min(amin);
      amax = warp_max(amax);
      // NaN a (a NaN DuPar or dlnB/ds) takes no part in the maximum, as the
      // reference's fabs(v) > max passes over NaN: no finite a, no sub-cycle
      double vmax = 0.0;
      for (int pass = 0; pass < 2 && amin <= amax; pass++) {
        const double a = pass ? amax : amin;
        for (int m = 1 + lane; m < M; m += 32) {
          const double vel = focus_vel(r.mugrid[m], a, b);
          const double vel_prev = focus_vel(r.mugrid[m - 1], a, b);
          vmax = fmax(vmax, fabs(m_(0.5, a_(vel, vel_prev))));
        }
      }
      vmax = warp_max(vmax);
      const double nsub = ceil(dt / (m_(0.9, r.dmu) / vmax));
      if (!(nsub <= (double)r.max_subcycles)) {
        if (ok && lane == 0)
          set_error(r, EPREM_GPU_ERR_SUBCYCLES, 2, (int)(g / N), (int)(g % N), -1, -1);
      } else {
        ns_f = (int)nsub;
      }
      if (!ok) ns_f = 0;
      c.dlnbds = (float)dlnbds;
      c.dupar = (float)dupar;
      c.b = (float)b;
      c.scale_f = (float)((dt / ns_f) / r.dmu);
    }
    if (r.use_change) {
      const double cool = (dlnn < 0) ? 1.0 - r.damp_cooling : 1.0;
      double vmax = 0.0;
      for (int pass = 0; pass < 2; pass++) {
        const double vi = r.ec[pass ? E - 1 : 0].vgrid_i;
        for (int m = lane; m < M; m += 32) {
          const double mu = r.mugrid[m];
          const double a = m_(-mu, dupar);
          const double bb =
              a_(m_(m_(mu, mu), s_(dlnn, dlnb)), m_(m_(0.5, s_(1.0, m_(mu, mu))), dlnb));
          vmax = fmax(vmax, fabs(m_(cool, a_(m_(a, vi), bb))));
        }
      }
      vmax = warp_max(vmax);
      const double nsub = ceil(dt / (m_(0.9, r.dlnp) / vmax));
      if (!(nsub <= (double)r.max_subcycles)) {
        if (ok && lane == 0)
          set_error(r, EPREM_GPU_ERR_SUBCYCLES, 3, (int)(g / N), (int)(g % N), -1, -1);
      } else {
        ns_c = (int)nsub;
      }
      if (!ok) ns_c = 0;
      c.cool = (float)cool;
      c.dlnb = (float)dlnb;
      c.dlnn = (float)dlnn;
      c.scale_c = (float)((dt / ns_c) / r.dlnp);
      if (lane < 2) {
        // ln seed = kb ln 2 + ln(seed 2^-kb), the integer part of log2 apart
        const double sv = seed_value(r, r.ec[lane ? E - 1 : 0], r.seed_radial[g]);
        const int kb = ilogb(sv);
        const float fb = (float)log(ldexp(sv, -kb));
        const float fo = __shfl_down_sync(0x3u, fb, 1);
        const int ko = __shfl_down_sync(0x3u, kb, 1);
        c.bc0 = fb;
        c.bc1 = fo;
        c.kbc0 = kb;
        c.kbc1 = ko;
      }
    }
    c.ns_f = ns_f;
    c.ns_c = ns_c;
    if (lane == 0) {
      r.coef32[g] = c;
      if (ok) {
        const unsigned long long EM = (unsigned long long)E * M * r.num_ep_steps;
        atomicMax(&s_max_f, ns_f);
        atomicMax(&s_max_c, ns_c);
        atomicAdd(&s_cs_f, (unsigned long long)ns_f * EM);
        atomicAdd(&s_cs_c, (unsigned long long)ns_c * EM);
      }
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (s_max_f) atomicMax(&r.status->max_focus, s_max_f);
    if (s_max_c) atomicMax(&r.status->max_change, s_max_c);
    if (s_cs_f) atomicAdd(&r.status->focus_cs, s_cs_f);
    if (s_cs_c) atomicAdd(&r.status->change_cs, s_cs_c);
  }
}

// ---- focusing: one (node, energy) row per thread ---------------------------
// A CTA's 128 rows are contiguous in f: they pass through shared memory
// (float4 loads and stores, rows padded to an odd pitch so each thread's row
// reads are free of bank conflicts) instead of one strided row per thread.
// FULL: M fills the register row (M = P), so every cell guard and the row /
// column split of the staging loops are known at compile time.
// One CTA's block blk of kFocusThreads rows of run r: the body of k_focus32
// and k_focus32_multi.
template <int P, bool FULL>
__device__ __forceinline__ void focus_block(const RunView &r, size_t blk) {
  extern __shared__ float tile[];  // [kFocusThreads][pitch]
  const int E = r.E, N = r.N;
  const int M = FULL ? P : r.M;
  const int pitch = M | 1;
  const size_t rows = (size_t)r.S * N * E;
  const size_t it0 = blk * kFocusThreads;
  const int nrows = (int)((rows - it0) < (size_t)kFocusThreads ? (rows - it0) : kFocusThreads);
  const int tid = threadIdx.x;
  float *base = reinterpret_cast<float *>(r.f) + it0 * M;
  const int nval = nrows * M;
  const float inv_m = 1.f / (float)M;  // row = floor((i + 1/2) / M), exact for i < 2^16
  // it0 * M is a multiple of 4 floats (it0 a multiple of 128): 16-byte aligned
  const int nvec = nval / 4;
  for (int v = tid; v < nvec; v += kFocusThreads) {
    const float4 x = reinterpret_cast<const float4 *>(base)[v];
    const float xs[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const int i = 4 * v + k, rr = FULL ? i / P : (int)(((float)i + 0.5f) * inv_m), cc = i - rr * M;
      tile[rr * pitch + cc] = xs[k];
    }
  }
  for (int i = 4 * nvec + tid; i < nval; i += kFocusThreads) {
    const int rr = (int)(((float)i + 0.5f) * inv_m), cc = i - rr * M;
    tile[rr * pitch + cc] = base[i];
  }
  __syncthreads();
  if (tid < nrows) {
    const size_t it = it0 + tid;
    const size_t g = it / E;
    const int e = (int)(it - g * E);
    const NodeCoef32 c = r.coef32[g];
    if (c.ok) {
      float *row = tile + tid * pitch;
      float fr[P];
#pragma unroll
      for (int m = 0; m < P; ++m)
        if (m < M) fr[m] = row[m];
      if (c.ns_f > 0) {
        const float v = r.ec[e].v32, vi = r.ec[e].vi32;
        const float a = -(v * c.dlnbds) - (2.f * vi) * c.dupar;
        const float b = c.b, sc = c.scale_f;
        // face m (between cells m-1 and m), m = 1..M-1: q = dt_sub/dmu times the
        // mean of the two cell velocities; flux = max(q,0) f[m-1] + min(q,0) f[m]
        float qp[P], qn[P];
        float vel_prev = 0.f;
#pragma unroll
        for (int m = 0; m < P; ++m) {
          qp[m] = qn[m] = 0.f;
          if (m < M) {
            const float mu = r.mugrid32[m];
            const float vel = 0.5f * (1.f - mu * mu) * (a + mu * b);
            if (m >= 1) {
              const float q = sc * 0.5f * (vel + vel_prev);
              // a NaN face speed reaches f, as in the reference's upwind flux
              qp[m] = q < 0.f ? 0.f : q;
              qn[m] = q > 0.f ? 0.f : q;
            }
            vel_prev = vel;
          }
        }
        for (int s = 0; s < c.ns_f; ++s) {
          float gprev = 0.f;
#pragma unroll
          for (int m = 0; m < P; ++m) {
            if (m < M) {
              float gnext = 0.f;
              if (m + 1 < M && m + 1 < P) gnext = fmaf(qn[m + 1], fr[m + 1], qp[m + 1] * fr[m]);
              fr[m] = fr[m] - (gnext - gprev);
              gprev = gnext;
            }
          }
        }
      }
      int code = 0;
#pragma unroll
      for (int m = 0; m < P; ++m) {
        if (m < M) {
          const float v = fr[m];
          if (bad_value(v, &code)) set_error(r, code, 2, (int)(g / N), (int)(g % N), e, m);
          row[m] = v < FLT_MIN ? FLT_MIN : v;
        }
      }
    }
  }
  __syncthreads();
  for (int v = tid; v < nvec; v += kFocusThreads) {
    float xs[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const int i = 4 * v + k, rr = FULL ? i / P : (int)(((float)i + 0.5f) * inv_m), cc = i - rr * M;
      xs[k] = tile[rr * pitch + cc];
    }
    reinterpret_cast<float4 *>(base)[v] = make_float4(xs[0], xs[1], xs[2], xs[3]);
  }
  for (int i = 4 * nvec + tid; i < nval; i += kFocusThreads) {
    const int rr = (int)(((float)i + 0.5f) * inv_m), cc = i - rr * M;
    base[i] = tile[rr * pitch + cc];
  }
}

// The run of CTA b among the runs of nv, whose first CTAs are off[0..n-1].
__device__ __forceinline__ int run_of_block(const int *off, int n, unsigned b) {
  int j = 0;
  while (j + 1 < n && (unsigned)off[j + 1] <= b) ++j;
  return j;
}

// Focusing over the rows of the runs of nv (one run, or the runs of one mu
// count of a lock-step ensemble): one launch, the same kernel either way, so
// a run's rows come out the same bit for bit.
template <int P, bool FULL>
__global__ void __launch_bounds__(kFocusThreads) k_focus32(const __grid_constant__ NodeRunViews nv) {
  const int j = run_of_block(nv.foff, nv.n, blockIdx.x);
  focus_block<P, FULL>(nv.v[j], blockIdx.x - (unsigned)nv.foff[j]);
}

// ---- adiabatic change: one (node, mu) column per thread --------------------
// A CTA holds whole nodes (npc = max(1, 128 / M) of them on npc * M threads)
// so that, after the sub-cycles, it can renormalise every row it writes.
// ln f of the columns lives in shared memory, [e][thread] (conflict-free), as
// delta = ln(stored value); row e's true ln f is delta + c_e with
// c_e = -fexp[e] ln 2.  The reference's flux-form update
//   l_e -= q_n l_a - q_p l_b   (a, b the upwind cells of faces e+1/2, e-1/2)
// is not invariant under a shift of l (q_n != q_p), so in delta it reads
//   delta_e -= q_n delta_a - q_p delta_b
//              + q_n (c_a - c_e) - q_p (c_b - c_e) + c_e (q_n - q_p),
// the exponent differences c_a - c_e formed from integers and
// q_n - q_p = dt_sub/dlnp cool am (1/v_{e+1} - 1/v_{e-1}) / 2 from the FP64
// difference of the grid (the bm part of the velocity cancels): no float
// rounding sees the size of ln f itself except through that small velocity
// difference.  The one-sided end cells and the Dirichlet seeds take the
// same exponent differences.  The change takes one or two sub-cycles per
// step, so its cost is the log / exp per cell (hardware approximations, ~1e-6
// relative on f).
// ln of a stored value relative to 2^kRowTop, where a normalised row's
// largest value lies, so that a row's leading cells have |ln| < 1 and keep
// float's relative precision in the flux-form update.  The value is scaled
// by an exact power of two first: by 2^-95 (__logf's absolute error on
// [0.5, 2], where the leading cells land, is about 4e-7), or for values
// more than 2^125 below the top, negligible in their row, by 2^31.  Taken
// of the stored value itself near 2^95, __logf's error and the rounding of
// a logarithm near 66 reached 1e-5 of f per conversion, a bias that the
// sub-steps of a run accumulated.  Values below FLT_MIN are the floor.
__device__ __forceinline__ float ln_rel(float v) {
  constexpr float kLn2 = 0.6931471805599453f;
  v = v < FLT_MIN ? FLT_MIN : v;
  const bool top = v >= 0x1p-30f;
  return __logf(v * (top ? 0x1p-95f : 0x1p31f)) + (top ? 0.f : -126.f * kLn2);
}
static_assert(kRowTop == 95, "ln_rel rescales by 2^-95");
// exp(l) * scale for l = ln_rel of a value and scale = 2^k, the row's
// exact power of two (0 below the float range): the exponential of the
// small relative logarithm, then one exact product; the far tail of a row
// (l below -80) takes 2^-64 into the exponential to stay above float
// underflow.
__device__ __forceinline__ float exp_rel(float l, float scale) {
  constexpr float kLn2 = 0.6931471805599453f;
  const bool near = l > -80.f;
  return __expf(near ? l : l + 64.f * kLn2) * (near ? scale : scale * 0x1p-64f);
}

// One CTA's block blk of npc nodes of run r: the body of k_change32 and
// k_change32_multi.
__device__ __forceinline__ void change_block(const RunView &r, int npc, size_t blk) {
  extern __shared__ float sm[];
  constexpr float kLn2 = 0.6931471805599453f;
  const int E = r.E, M = r.M;
  const int T = npc * M;  // live threads of the CTA
  const int tid = threadIdx.x;
  const int j = tid / M, m = tid - (tid / M) * M;
  const size_t SN = (size_t)r.S * r.N;
  const size_t g = blk * npc + j;
  float *lnf = sm;                                             // [E][T]
  int *xs = reinterpret_cast<int *>(sm + (size_t)E * T);     // [npc][E] row exponents
  int *sh = xs + npc * E;                                      // [npc][E] renormalising shifts
  float *sc = reinterpret_cast<float *>(sh + npc * E);         // [npc][E] 2^(sh + kRowTop)
  float *dnl = sc + npc * E;   // [npc][E] (x_e - x_{e+1}) ln 2
  float *xd = dnl + npc * E;   // [npc][E] x_e ln 2 (1/v_{e+1} - 1/v_{e-1})
  float *vw = xd + npc * E;    // [E] 1/v_e + 1/v_{e+1}: face e+1's sum of the two cells' 1/v
  // the rows' exponents less kRowTop: ln f = lnf - xs ln 2 with lnf the ln of
  // a stored value relative to 2^kRowTop (see ln_rel)
  for (int i = tid; i < npc * E; i += blockDim.x) {
    const size_t gg = blk * npc + i / E;
    xs[i] = (gg < SN ? r.fexp[gg * E + i % E] : 0) - kRowTop;
  }
  for (int e = tid; e < E; e += blockDim.x)
    vw[e] = e + 1 < E ? r.ec[e].vi32 + r.ec[e + 1].vi32 : 0.f;
  __syncthreads();
  // each row's exponent terms of the flux form, once per node and energy
  for (int i = tid; i < npc * E; i += blockDim.x) {
    const int e = i % E;
    dnl[i] = e + 1 < E ? (float)(xs[i] - xs[i + 1]) * kLn2 : 0.f;
    xd[i] = ((float)xs[i] * kLn2) * r.ec[e].dvi32;
  }
  bool ok = false;
  NodeCoef32 c{};
  if (tid < T && g < SN) {
    c = r.coef32[g];
    ok = c.ok != 0;  // the spawn node is not changed
  }
  float *col = reinterpret_cast<float *>(r.f) + (ok ? g : 0) * E * M + m;  // stride M
  float *fc = lnf + tid;                                                    // stride T
  if (ok)
    for (int e = 0; e < E; ++e) fc[e * T] = ln_rel(col[e * M]);
  __syncthreads();
  if (ok && c.ns_c > 0) {
    const int *x = xs + j * E;
    const float *dn_j = dnl + j * E, *xd_j = xd + j * E;
    const float mu = r.mugrid32[m];
    const float am = -mu * c.dupar;
    const float bm = mu * mu * (c.dlnn - c.dlnb) + 0.5f * (1.f - mu * mu) * c.dlnb;
    const float cool = c.cool, sc = c.scale_c;
    const float hq = sc * 0.5f * cool * am;  // q_n - q_p = hq (1/v_{e+1} - 1/v_{e-1})
    // the seeds relative to the first and last rows' exponents
    const float bc0 = c.bc0 + (float)(c.kbc0 + x[0]) * kLn2;
    const float bc1 = c.bc1 + (float)(c.kbc1 + x[E - 1]) * kLn2;
    const float sch = sc * 0.5f;
    // face e+1 (between energies e and e+1): q = dt_sub/dlnp times the mean of
    // the two cell velocities cool (am/v + bm) = qa (1/v_e + 1/v_{e+1}) + qb
    const float qa = sch * cool * am, qb = sch * cool * (2.f * bm);
    for (int s = 0; s < c.ns_c; ++s) {
      const float q1 = qa * vw[0] + qb;
      const float f0 = fc[0], f1 = fc[T];
      float dprev = dn_j[0];  // c_1 - c_0
      float gprev = q1 * (q1 >= 0.f ? f0 : f1);
      float cprev = q1 >= 0.f ? q1 * dprev : 0.f;  // -q_p (c_b - c_e) of the next cell
      const float d0 = (q1 <= 0.f) ? q1 * (f1 - f0 + dprev) : q1 * (f0 - bc0);
      float fold_prev = f0;
      fc[0] = f0 - d0;
      float qcur = q1, fe = f1;
      for (int e = 1; e < E - 1; ++e) {
        const float qq = qa * vw[e] + qb;
        const float fn = fc[(e + 1) * T];
        const float dn = dn_j[e];  // c_{e+1} - c_e
        const float qdn = qq * dn;
        const bool up = qq >= 0.f;
        const float gnext = qq * (up ? fe : fn);
        // c_e's share of the divergence term: x_e ln2 hq (1/v_{e+1} - 1/v_{e-1})
        const float corr = (up ? 0.f : qdn) + cprev - hq * xd_j[e];
        fold_prev = fe;
        fc[e * T] = fe - (gnext - gprev) - corr;
        gprev = gnext;
        cprev = up ? qdn : 0.f;
        qcur = qq;
        fe = fn;
        dprev = dn;
      }
      // last energy (e = E-1): upwind from below, or the Dirichlet seed above
      const float dl = (qcur >= 0.f) ? qcur * (fe - fold_prev + dprev) : qcur * (bc1 - fe);
      fc[(E - 1) * T] = fe - dl;
    }
  }
  __syncthreads();
  // each row's new exponent: its largest value to [2^kRowTop, 2^(kRowTop+1))
  if (ok)
    for (int e = m; e < E; e += M) {
      const float *rowp = lnf + (size_t)e * T + j * M;
      float mx = rowp[0];
      for (int mm = 1; mm < M; ++mm) mx = fmaxf(mx, rowp[mm]);
      const float l2 = fminf(fmaxf(floorf(mx * 1.4426950408889634f), -1.0e6f), 1.0e6f);
      const int x0 = xs[j * E + e] + kRowTop;
      const int d = clamp_exp(x0 - (int)l2) - x0;
      sh[j * E + e] = d;
      sc[j * E + e] = d + kRowTop >= -126 ? pow2f(min(d + kRowTop, 127)) : 0.f;
    }
  __syncthreads();
  if (ok) {
    int code = 0;
    for (int e = 0; e < E; ++e) {
      const float v = exp_rel(fc[e * T], sc[j * E + e]);
      if (bad_value(v, &code)) set_error(r, code, 3, (int)(g / r.N), (int)(g % r.N), e, m);
      col[e * M] = v < FLT_MIN ? FLT_MIN : v;
    }
    for (int e = m; e < E; e += M)
      r.fexp[g * E + e] = (short)(xs[j * E + e] + kRowTop + sh[j * E + e]);
  }
}

// The change over the nodes of the runs of nv, as k_focus32 over their rows.
__global__ void __launch_bounds__(kChangeThreads)
    k_change32(const __grid_constant__ NodeRunViews nv, int npc) {
  const int j = run_of_block(nv.coff, nv.n, blockIdx.x);
  change_block(nv.v[j], npc, blockIdx.x - (unsigned)nv.coff[j]);
}

// Row lengths the focusing kernel is built for (20: the CPU-runnable case's
// mu count, with compile-time cell guards).
static int bucket(int n) {
  for (int b : {8, 16, 20, 24, 32, 40, 48, 56, 64})
    if (n <= b) return b;
  return 0;
}

int plan_node32(int E, int M, NodePlan *plan) {
  if (E < 2 || M < 2 || !bucket(E) || !bucket(M)) return EPREM_GPU_ERR_ARG;
  plan->pmax = bucket(M);  // focusing row length
  plan->pcol = E;          // change column length (shared memory)
  plan->nodes = 1;
  plan->threads = kFocusThreads;
  plan->smem = 0;
  return 0;
}

int launch_node32_setup(const RunView &r, cudaStream_t st, uint64_t *launches) {
  const size_t SN = (size_t)r.S * r.N;
  const unsigned blocks = (unsigned)((SN + kSetupWarps - 1) / kSetupWarps);
  k_node32_setup<<<blocks, kSetupWarps * 32, 0, st>>>(r);
  *launches += 1;
  return cudaGetLastError() == cudaSuccess ? 0 : EPREM_GPU_ERR_CUDA;
}

static int change_npc(int M) { return M >= kChangeThreads ? 1 : kChangeThreads / M; }
static size_t change_smem(int E, int M) {
  const int npc = change_npc(M);
  return (size_t)E * npc * M * sizeof(float) + 5 * (size_t)npc * E * sizeof(int) +
         (size_t)E * sizeof(float);
}

void node32_blocks(const RunView &r, int *focus_blocks, int *change_blocks) {
  const size_t rows = (size_t)r.S * r.N * r.E, SN = (size_t)r.S * r.N;
  const int npc = change_npc(r.M);
  *focus_blocks = (int)((rows + kFocusThreads - 1) / kFocusThreads);
  *change_blocks = (int)((SN + npc - 1) / npc);
}

// nv's runs share M (and so P and npc)
template <int P>
static void launch_focus_t(const NodeRunViews &nv, cudaStream_t st) {
  const int M = nv.v[0].M;
  const size_t smem = (size_t)kFocusThreads * (M | 1) * sizeof(float);
  if (M == P)
    k_focus32<P, true><<<nv.foff[nv.n], kFocusThreads, smem, st>>>(nv);
  else
    k_focus32<P, false><<<nv.foff[nv.n], kFocusThreads, smem, st>>>(nv);
}

static void launch_change(const NodeRunViews &nv, cudaStream_t st) {
  const int M = nv.v[0].M, npc = change_npc(M);
  size_t smem = 0;
  for (int i = 0; i < nv.n; i++) {
    const size_t b = change_smem(nv.v[i].E, M);
    smem = b > smem ? b : smem;
  }
  if (smem > 48 * 1024)
    cudaFuncSetAttribute(k_change32, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k_change32<<<nv.coff[nv.n], kChangeThreads, smem, st>>>(nv, npc);
}

#define EPREM_P_SWITCH(p, F, ...)      \
  switch (p) {                         \
    case 8: F<8>(__VA_ARGS__); break;   \
    case 16: F<16>(__VA_ARGS__); break; \
    case 20: F<20>(__VA_ARGS__); break; \
    case 24: F<24>(__VA_ARGS__); break; \
    case 32: F<32>(__VA_ARGS__); break; \
    case 40: F<40>(__VA_ARGS__); break; \
    case 48: F<48>(__VA_ARGS__); break; \
    case 56: F<56>(__VA_ARGS__); break; \
    default: F<64>(__VA_ARGS__); break; \
  }

int launch_node32_multi(const NodePlan &pl, const NodeRunViews &nv, cudaStream_t st,
                        uint64_t *launches) {
  if (nv.n <= 0 || nv.n > kMultiRuns) return EPREM_GPU_ERR_ARG;
  EPREM_P_SWITCH(pl.pmax, launch_focus_t, nv, st);
  launch_change(nv, st);
  *launches += 2;
  return cudaGetLastError() == cudaSuccess ? 0 : EPREM_GPU_ERR_CUDA;
}

int launch_node32(const RunView &r, const NodePlan &pl, cudaStream_t st, uint64_t *launches) {
  NodeRunViews nv;
  nv.v[0] = r;
  nv.n = 1;
  nv.foff[0] = nv.coff[0] = 0;
  node32_blocks(r, &nv.foff[1], &nv.coff[1]);
  if (r.use_focus) {
    EPREM_P_SWITCH(pl.pmax, launch_focus_t, nv, st);
    *launches += 1;
  }
  if (r.use_change) {
    launch_change(nv, st);
    *launches += 1;
  }
  return cudaGetLastError() == cudaSuccess ? 0 : EPREM_GPU_ERR_CUDA;
}

}  // namespace eprem
