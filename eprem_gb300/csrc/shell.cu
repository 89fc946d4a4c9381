// shell.cu -- cross-field (shell) diffusion: DiffuseShellData
// (src/energeticParticles.c:419-554) with the perpendicular neighbour lengths
// of ShellData (:254-413).
//
// Each sub-step, every node k >= 1 of every stream hands a fraction
//   del = min(dt * 0.33333333 * mfp * v * kperxkpar / (dlPer^2 + 1e-33), 0.025)
// of its f to each of its four NEWS neighbours on the same shell and loses
// their sum.  The reference accumulates all hand-overs of one (shell, energy)
// in deltaShell, sources in ascending stream order and, per source, north,
// east, west, south and then the source's own loss, and adds deltaShell to f
// afterwards.  Here each target cell gathers the same terms in the same order
// from a per-target list built on the host (source stream, direction), so the
// FP64 form reproduces the reference's sums bit for bit; this file is built
// without fused multiply-adds for that reason.
//
// Node positions and B do not change inside one update, so the lengths and
// fractions (k_shell_coef) are formed once per call for all its sub-steps.
#include <algorithm>

#include "common.cuh"
#include "kernels.h"

namespace eprem {

// One thread per node (s, k >= 1): ShellData's four lengths, then per energy
// the four fractions and their sum, slice-major so that one (node, energy)
// slice's fractions sit together: del[((k*E + e)*S + s)*5 + {0..3, 4}].
// Formed in double, stored as the f type (float in the FP32 form, whose
// diffusion then runs without FP64 instructions).
template <typename Real>
__global__ void k_shell_coef(RunView r, const int *news, double kperxkpar, Real *del) {
  const size_t SN = (size_t)r.S * r.N;
  const double *rx = node_field(r, EPREM_NODE_RX), *ry = node_field(r, EPREM_NODE_RY),
               *rz = node_field(r, EPREM_NODE_RZ), *bm = node_field(r, EPREM_NODE_BMAG),
               *bx = node_field(r, EPREM_NODE_BVEC_X), *by = node_field(r, EPREM_NODE_BVEC_Y),
               *bz = node_field(r, EPREM_NODE_BVEC_Z);
  const double rs = r.r_scale;
  for (size_t g = blockIdx.x * (size_t)blockDim.x + threadIdx.x; g < SN;
       g += (size_t)gridDim.x * blockDim.x) {
    const int s = (int)(g / r.N), k = (int)(g % r.N);
    if (k == 0) continue;
    const double x = __dmul_rn(rx[g], rs), y = __dmul_rn(ry[g], rs), z = __dmul_rn(rz[g], rs);
    const double ebx = bx[g] / bm[g], eby = by[g] / bm[g], ebz = bz[g] / bm[g];
    double dlper[4];
    for (int d = 0; d < 4; d++) {
      const size_t o = (size_t)news[s * 4 + d] * r.N + k;
      double ex = __dsub_rn(__dmul_rn(rx[o], rs), x), ey = __dsub_rn(__dmul_rn(ry[o], rs), y),
             ez = __dsub_rn(__dmul_rn(rz[o], rs), z);
      const double dl =
          sqrt(__dadd_rn(__dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey)), __dmul_rn(ez, ez)));
      ex = ex / dl;
      ey = ey / dl;
      ez = ez / dl;
      const double dot =
          __dadd_rn(__dadd_rn(__dmul_rn(ex, ebx), __dmul_rn(ey, eby)), __dmul_rn(ez, ebz));
      dlper[d] = __dmul_rn(dl, sqrt(__dsub_rn(1.0, __dmul_rn(dot, dot))));
    }
    const double mf = r.mfp_node[g];
    for (int e = 0; e < r.E; e++) {
      const double mfp = __dmul_rn(r.ec[e].rig_lamo, mf);
      const double dt_kper =
          __dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(r.dt, 0.33333333), mfp), r.ec[e].vgrid), kperxkpar);
      Real *out = del + (((size_t)k * r.E + e) * r.S + s) * 5;
      double sum = 0.0;
      Real rsum = Real(0);
      for (int d = 0; d < 4; d++) {
        double v = dt_kper / __dadd_rn(__dmul_rn(dlper[d], dlper[d]), kVerySmall);
        if (v > 0.025) v = 0.025;
        out[d] = (Real)v;
        sum = d == 0 ? v : __dadd_rn(sum, v);
        rsum = d == 0 ? out[d] : rsum + out[d];
      }
      // FP64: the reference's sum.  FP32: the sum of the rounded fractions in
      // the same order, so that a node's loss is its neighbours' gains up to
      // the rounding of the accumulation
      out[4] = sizeof(Real) == 8 ? (Real)sum : rsum;
    }
  }
}

// DriftShellData's hand-over fractions (src/energeticParticles.c:561-801):
// one thread per node (s, k >= 1); per energy the drift velocity of
// driftVelocity (:210-246: drift_factor times curl(B)/B^2, to Cartesian by
// sphToCartVector, src/geometry.c:89-125) and per NEWS direction
// vdp = (v_d . (r_nbr - r)) rScale / dl with dl the neighbour distance of
// ShellData (:254-413); del = min(vdp dt / dl, 0.025) where vdp > 0, else 0
// (no hand-over).  del[((k*E + e)*S + s)*4 + d], in the f type.  The
// reference's expressions and order, no fused multiply-adds.
template <typename Real>
__global__ void k_drift_coef(RunView r, const int *news, Real *del) {
  const size_t SN = (size_t)r.S * r.N;
  const double *rx = node_field(r, EPREM_NODE_RX), *ry = node_field(r, EPREM_NODE_RY),
               *rz = node_field(r, EPREM_NODE_RZ);
  const double rs = r.r_scale;
  for (size_t g = blockIdx.x * (size_t)blockDim.x + threadIdx.x; g < SN;
       g += (size_t)gridDim.x * blockDim.x) {
    const int s = (int)(g / r.N), k = (int)(g % r.N);
    if (k == 0) continue;
    const double x = rx[g], y = ry[g], z = rz[g];
    const double xs = __dmul_rn(x, rs), ys = __dmul_rn(y, rs), zs = __dmul_rn(z, rs);
    double en[4][3], dl[4];
    for (int d = 0; d < 4; d++) {
      const size_t o = (size_t)news[s * 4 + d] * r.N + k;
      const double ex = __dsub_rn(__dmul_rn(rx[o], rs), xs), ey = __dsub_rn(__dmul_rn(ry[o], rs), ys),
                   ez = __dsub_rn(__dmul_rn(rz[o], rs), zs);
      dl[d] = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey)), __dmul_rn(ez, ez)));
      en[d][0] = __dsub_rn(rx[o], x);
      en[d][1] = __dsub_rn(ry[o], y);
      en[d][2] = __dsub_rn(rz[o], z);
    }
    const double cr = r.curl[g], ct = r.curl[r.node_stride + g], cp = r.curl[2 * r.node_stride + g];
    const double rmag = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z)));
    const double rho2 = __dsub_rn(__dmul_rn(rmag, rmag), __dmul_rn(z, z));
    const bool axis = __dsub_rn(rmag, fabs(z)) < kVerySmall;
    for (int e = 0; e < r.E; e++) {
      const double fac = r.ec[e].drift_factor;
      const double vr = __dmul_rn(fac, cr), vt = __dmul_rn(fac, ct), vp = __dmul_rn(fac, cp);
      double vx = 0.0, vy = 0.0;
      if (!axis) {
        vx = __dsub_rn(__dadd_rn(__dmul_rn(x / rmag, vr), __dmul_rn(__dmul_rn(x, z) / __dmul_rn(rmag, sqrt(rho2)), vt)),
                       __dmul_rn(y / sqrt(rho2), vp));
        vy = __dadd_rn(__dadd_rn(__dmul_rn(y / rmag, vr), __dmul_rn(__dmul_rn(y, z) / __dmul_rn(rmag, sqrt(rho2)), vt)),
                       __dmul_rn(x / sqrt(rho2), vp));
      }
      const double vz = __dsub_rn(__dmul_rn(z / rmag, vr), __dmul_rn(sqrt(rho2) / rmag, vt));
      Real *out = del + (((size_t)k * r.E + e) * r.S + s) * 4;
      for (int d = 0; d < 4; d++) {
        const double dot = __dadd_rn(__dadd_rn(__dmul_rn(vx, en[d][0]), __dmul_rn(vy, en[d][1])),
                                     __dmul_rn(vz, en[d][2]));
        const double vdp = __dmul_rn(dot, rs) / dl[d];
        double dd = 0.0;
        if (vdp > 0.0) {
          dd = __dmul_rn(vdp, r.dt) / dl[d];
          if (dd > 0.025) dd = 0.025;
        }
        out[d] = (Real)dd;
      }
    }
  }
}

__device__ __forceinline__ double sd_fma(double a, double b, double acc) {
  return __dadd_rn(acc, __dmul_rn(a, b));
}
__device__ __forceinline__ double sd_fms(double a, double b, double acc) {
  return __dsub_rn(acc, __dmul_rn(a, b));
}
__device__ __forceinline__ float sd_fma(float a, float b, float acc) { return __fmaf_rn(a, b, acc); }
__device__ __forceinline__ float sd_fms(float a, float b, float acc) { return __fmaf_rn(-a, b, acc); }

// NaN or Inf, by the exponent bits (no floating-point instruction)
__device__ __forceinline__ bool nonfinite(double v) {
  return (__double_as_longlong(v) & 0x7ff0000000000000LL) == 0x7ff0000000000000LL;
}
__device__ __forceinline__ bool nonfinite(float v) {
  return (__float_as_uint(v) & 0x7f800000u) == 0x7f800000u;
}

// V consecutive values of f (V = 1 or 2: one 8- or 16-byte access)
template <int V, typename Real>
__device__ __forceinline__ void ld_vec(const Real *p, Real (&x)[V]) {
  if constexpr (V == 1) {
    x[0] = __ldg(p);
  } else if constexpr (sizeof(Real) == 4) {
    const float2 t = __ldg(reinterpret_cast<const float2 *>(p));
    x[0] = t.x, x[1] = t.y;
  } else {
    const double2 t = __ldg(reinterpret_cast<const double2 *>(p));
    x[0] = t.x, x[1] = t.y;
  }
}
template <int V, typename Real>
__device__ __forceinline__ void st_vec(Real *p, const Real (&x)[V]) {
  if constexpr (V == 1) {
    p[0] = x[0];
  } else if constexpr (sizeof(Real) == 4) {
    *reinterpret_cast<float2 *>(p) = make_float2(x[0], x[1]);
  } else {
    *reinterpret_cast<double2 *>(p) = make_double2(x[0], x[1]);
  }
}

// One (node, energy) slice of all streams per block at a time (blocks stride
// over the N*E slices), so the neighbours' reads of a slice come from L2 and
// f crosses HBM once each way.  Writes the new f to out (node 0 copied
// unchanged); the caller then makes out the run's f.  ent[s*L + p] = source
// stream * 8 + direction (0..3 north..south, 4 the target's own loss), -1
// past the end of the target's list.  A thread takes V adjacent mu cells
// (V = 2 when M is even: the list and fractions are read once for both) at
// two places of the slice blockDim apart ((stream, mu) stepped by counters,
// no divisions), and issues every load of a chunk of C list entries before
// the ordered sums.
// FP32 form: the terms of a target row come from rows with their own
// exponents.  The new row's exponent is the target's, lowered where a gain
// could otherwise leave the float range: a source row's values lie below
// 2^(kRowTop+7) in its own scale (normalised, then focused at most M-fold),
// so a gain a f_i stays below 2^120 in an exponent no higher than
// fexp_i + 17 - log2(a).  Every term is taken to that exponent (exact powers
// of two) before the sum; xout receives it.
// DRIFT: the same gather for DriftShellData, whose lists hold a loss per
// direction (code = source * 8 + 4 + direction, right after that direction's
// gain) with the fractions four per source ([N][E][S][4]).
template <typename Real, int C, int V, bool DRIFT>
__global__ void __launch_bounds__(256, sizeof(Real) == 4 ? 4 : 2)
    k_shell_diffuse(RunView r, const int *__restrict__ ent, int L, const Real *__restrict__ del,
                    Real *__restrict__ out, short *__restrict__ xout) {
  constexpr int NCOEF = DRIFT ? 4 : 5;  // fractions per source
  auto coef_of = [](int code) { return DRIFT ? (code & 3) : (code & 7); };
  auto is_gain = [](int code) { return (code & 7) < 4; };
  const Real *__restrict__ f = static_cast<const Real *>(r.f);
  const int M = r.M, S = r.S, E = r.E;
  const int MV = M / V;      // V-cell groups per row
  const int groups = S * MV;  // of one slice
  const size_t per_stream = (size_t)r.N * E * M;
  const int nslices = r.N * E;
  const int inc_s = blockDim.x / MV, inc_m = blockDim.x % MV;
  const int s_first = threadIdx.x / MV, m_first = threadIdx.x % MV;
  for (int sl = blockIdx.x; sl < nslices; sl += gridDim.x) {
    const int k = sl / E, e = sl - (sl / E) * E;
    const size_t row = (size_t)sl * M;                 // (k*E + e)*M within a stream
    const Real *__restrict__ dsl = del + (size_t)sl * S * NCOEF;
    int s0 = s_first, m0 = m_first;
    for (int c = threadIdx.x; c < groups; c += 2 * blockDim.x) {
      int s[2], m[2];
      s[0] = s0;
      m[0] = m0;
      s[1] = s0 + inc_s;
      m[1] = m0 + inc_m;
      if (m[1] >= MV) {
        m[1] -= MV;
        s[1]++;
      }
      const bool ok1 = c + (int)blockDim.x < groups;
      if (!ok1) s[1] = s[0], m[1] = m[0];
      s0 = s[1] + inc_s;  // the next pair starts blockDim past the second group
      m0 = m[1] + inc_m;
      if (m0 >= MV) {
        m0 -= MV;
        s0++;
      }
      Real acc[2][V];
#pragma unroll
      for (int u = 0; u < 2; u++)
#pragma unroll
        for (int j = 0; j < V; j++) acc[u][j] = Real(0);
      int xt[2] = {0, 0}, xn[2] = {0, 0};  // FP32 form: target's exponent, new exponent
      if constexpr (sizeof(Real) == 4) {
#pragma unroll
        for (int u = 0; u < 2; u++) {
          xt[u] = r.fexp[((size_t)s[u] * r.N + k) * E + e];
          int b = xt[u];
          for (int p = 0; k > 0 && p < L; ++p) {
            const int cd = __ldg(ent + s[u] * L + p);
            if (cd < 0 || !is_gain(cd)) continue;
            const float a = (float)__ldg(dsl + (cd >> 3) * NCOEF + coef_of(cd));
            if (!(a > 0.f)) continue;
            const int xi = r.fexp[((size_t)(cd >> 3) * r.N + k) * E + e];
            b = min(b, xi + 17 - ilogb_f(a));
          }
          xn[u] = b < xt[u] ? clamp_exp(b) : xt[u];
        }
      }
      for (int p0 = 0; k > 0 && p0 < L; p0 += C) {
        int code[2][C];
        Real a[2][C], fi[2][C][V];
#pragma unroll
        for (int u = 0; u < 2; u++)
#pragma unroll
          for (int q = 0; q < C; q++)
            code[u][q] = p0 + q < L ? __ldg(ent + s[u] * L + p0 + q) : -1;
#pragma unroll
        for (int u = 0; u < 2; u++)
#pragma unroll
          for (int q = 0; q < C; q++) {
            a[u][q] = Real(0);
#pragma unroll
            for (int j = 0; j < V; j++) fi[u][q][j] = Real(0);
            if (code[u][q] >= 0) {
              const int i = code[u][q] >> 3;
              a[u][q] = __ldg(dsl + i * NCOEF + coef_of(code[u][q]));
              ld_vec<V>(f + (size_t)i * per_stream + row + (size_t)m[u] * V, fi[u][q]);
              if constexpr (sizeof(Real) == 4)  // the source row taken to the new exponent
                a[u][q] = ldexp_f(a[u][q], xn[u] - r.fexp[((size_t)i * r.N + k) * E + e]);
            }
          }
#pragma unroll
        for (int u = 0; u < 2; u++)
#pragma unroll
          for (int q = 0; q < C; q++)
            if (code[u][q] >= 0) {
              const bool gain = is_gain(code[u][q]);
#pragma unroll
              for (int j = 0; j < V; j++)
                acc[u][j] = gain ? sd_fma(a[u][q], fi[u][q][j], acc[u][j])
                                 : sd_fms(a[u][q], fi[u][q][j], acc[u][j]);
            }
      }
#pragma unroll
      for (int u = 0; u < 2; u++) {
        if (u == 1 && !ok1) break;
        const size_t gi = (size_t)s[u] * per_stream + row + (size_t)m[u] * V;
        Real v[V];
        ld_vec<V>(f + gi, v);
        if constexpr (sizeof(Real) == 4) {
          if (xn[u] != xt[u])
#pragma unroll
            for (int j = 0; j < V; j++) v[j] = ldexp_f(v[j], xn[u] - xt[u]);
          if (m[u] == 0) xout[((size_t)s[u] * r.N + k) * E + e] = (short)xn[u];
        }
        if (k > 0) {
#pragma unroll
          for (int j = 0; j < V; j++) {
            v[j] = v[j] + acc[u][j];
            if (nonfinite(v[j]))
              set_error(r, isnan(v[j]) ? EPREM_GPU_ERR_NAN : EPREM_GPU_ERR_INF, DRIFT ? 7 : 6,
                        s[u], k, e, m[u] * V + j);
          }
        }
        st_vec<V>(out + gi, v);
      }
    }
  }
}

int launch_shell_coef(const RunView &r, const int *news, double kperxkpar, void *del,
                      cudaStream_t st, uint64_t *launches) {
  const size_t SN = (size_t)r.S * r.N;
  const int blocks = (int)std::min<size_t>((SN + 127) / 128, 152 * 8);
  if (r.precision == EPREM_FP32)
    k_shell_coef<float><<<blocks, 128, 0, st>>>(r, news, kperxkpar, (float *)del);
  else
    k_shell_coef<double><<<blocks, 128, 0, st>>>(r, news, kperxkpar, (double *)del);
  ++*launches;
  return cudaPeekAtLastError() == cudaSuccess ? 0 : EPREM_GPU_ERR_CUDA;
}

template <typename Real, bool DRIFT>
static void shell_diffuse_as(const RunView &r, const int *ent, int L, const void *del,
                             void *out, short *xout, int blocks, cudaStream_t st) {
  const Real *d = (const Real *)del;
  Real *o = (Real *)out;
  const bool pairs = r.M % 2 == 0;
  if (L <= 5 && pairs)
    k_shell_diffuse<Real, 5, 2, DRIFT><<<blocks, 256, 0, st>>>(r, ent, L, d, o, xout);
  else if (L <= 5)
    k_shell_diffuse<Real, 5, 1, DRIFT><<<blocks, 256, 0, st>>>(r, ent, L, d, o, xout);
  else if (pairs)
    k_shell_diffuse<Real, 8, 2, DRIFT><<<blocks, 256, 0, st>>>(r, ent, L, d, o, xout);
  else
    k_shell_diffuse<Real, 8, 1, DRIFT><<<blocks, 256, 0, st>>>(r, ent, L, d, o, xout);
}

int launch_shell_diffuse(const RunView &r, const int *ent, int L, const void *del, void *out,
                         short *xout, cudaStream_t st, uint64_t *launches, bool drift) {
  const int blocks = std::min(r.N * r.E, 152 * 8);
  if (r.precision == EPREM_FP32) {
    if (drift)
      shell_diffuse_as<float, true>(r, ent, L, del, out, xout, blocks, st);
    else
      shell_diffuse_as<float, false>(r, ent, L, del, out, xout, blocks, st);
  } else {
    if (drift)
      shell_diffuse_as<double, true>(r, ent, L, del, out, nullptr, blocks, st);
    else
      shell_diffuse_as<double, false>(r, ent, L, del, out, nullptr, blocks, st);
  }
  ++*launches;
  return cudaPeekAtLastError() == cudaSuccess ? 0 : EPREM_GPU_ERR_CUDA;
}

int launch_drift_coef(const RunView &r, const int *news, void *del, cudaStream_t st,
                      uint64_t *launches) {
  const size_t SN = (size_t)r.S * r.N;
  const int blocks = (int)std::min<size_t>((SN + 127) / 128, 152 * 8);
  if (r.precision == EPREM_FP32)
    k_drift_coef<float><<<blocks, 128, 0, st>>>(r, news, (float *)del);
  else
    k_drift_coef<double><<<blocks, 128, 0, st>>>(r, news, (double *)del);
  ++*launches;
  return cudaPeekAtLastError() == cudaSuccess ? 0 : EPREM_GPU_ERR_CUDA;
}

}  // namespace eprem
