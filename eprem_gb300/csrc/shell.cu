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
__global__ void k_shell_coef(RunView r, const int *news, double kperxkpar, double *del) {
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
      double *out = del + (((size_t)k * r.E + e) * r.S + s) * 5;
      double sum = 0.0;
      for (int d = 0; d < 4; d++) {
        double v = dt_kper / __dadd_rn(__dmul_rn(dlper[d], dlper[d]), kVerySmall);
        if (v > 0.025) v = 0.025;
        out[d] = v;
        sum = d == 0 ? v : __dadd_rn(sum, v);
      }
      out[4] = sum;
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

// All cells, ordered (k, e, stream, mu): one (node, energy) slice of all
// streams is in flight at a time, so the neighbours' reads of a slice come
// from L2 and f crosses HBM once each way.  Writes the new f to out (node 0
// copied unchanged); the caller then makes out the run's f.  ent[s*L + p] =
// source stream * 8 + direction (0..3 north..south, 4 the target's own loss),
// -1 past the end of the target's list.  Each thread takes two cells a
// stride apart and issues every load of a chunk of C list entries before the
// ordered sums, so a warp waits once per chunk rather than once per term.
template <typename Real, int C>
__global__ void __launch_bounds__(256) k_shell_diffuse(RunView r, const int *__restrict__ ent,
                                                       int L, const double *__restrict__ del,
                                                       Real *__restrict__ out) {
  const Real *__restrict__ f = static_cast<const Real *>(r.f);
  const size_t M = r.M, S = r.S, E = r.E;
  const size_t per_stream = (size_t)r.N * E * M;
  const size_t total = (size_t)r.N * E * S * M;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t t0 = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t0 < total; t0 += 2 * stride) {
    int s[2], k[2], e[2], m[2];
    bool ok[2];
#pragma unroll
    for (int u = 0; u < 2; u++) {
      const size_t t = t0 + u * stride;
      ok[u] = t < total;
      const size_t tc = ok[u] ? t : t0;
      m[u] = (int)(tc % M);
      size_t q = tc / M;
      s[u] = (int)(q % S);
      q /= S;
      e[u] = (int)(q % E);
      k[u] = (int)(q / E);
    }
    Real acc[2] = {Real(0), Real(0)};
    for (int p0 = 0; p0 < L; p0 += C) {
      int code[2][C];
      Real a[2][C], fi[2][C];
#pragma unroll
      for (int u = 0; u < 2; u++)
#pragma unroll
        for (int q = 0; q < C; q++)
          code[u][q] = (k[u] > 0 && p0 + q < L) ? __ldg(ent + (size_t)s[u] * L + p0 + q) : -1;
#pragma unroll
      for (int u = 0; u < 2; u++)
#pragma unroll
        for (int q = 0; q < C; q++) {
          a[u][q] = Real(0);
          fi[u][q] = Real(0);
          if (code[u][q] >= 0) {
            const int i = code[u][q] >> 3, d = code[u][q] & 7;
            a[u][q] = (Real)__ldg(del + (((size_t)k[u] * E + e[u]) * S + i) * 5 + d);
            fi[u][q] = __ldg(f + (size_t)i * per_stream + ((size_t)k[u] * E + e[u]) * M + m[u]);
          }
        }
#pragma unroll
      for (int u = 0; u < 2; u++)
#pragma unroll
        for (int q = 0; q < C; q++)
          if (code[u][q] >= 0)
            acc[u] = (code[u][q] & 7) < 4 ? sd_fma(a[u][q], fi[u][q], acc[u])
                                          : sd_fms(a[u][q], fi[u][q], acc[u]);
    }
#pragma unroll
    for (int u = 0; u < 2; u++) {
      if (!ok[u]) continue;
      const size_t gi = (size_t)s[u] * per_stream + ((size_t)k[u] * E + e[u]) * M + m[u];
      const Real fo = f[gi];
      if (k[u] == 0) {
        out[gi] = fo;
        continue;
      }
      const Real v = fo + acc[u];
      out[gi] = v;
      if (isnan((double)v) || isinf((double)v))
        set_error(r, isnan((double)v) ? EPREM_GPU_ERR_NAN : EPREM_GPU_ERR_INF, 6, s[u], k[u],
                  e[u], m[u]);
    }
  }
}

int launch_shell_coef(const RunView &r, const int *news, double kperxkpar, double *del,
                      cudaStream_t st, uint64_t *launches) {
  const size_t SN = (size_t)r.S * r.N;
  const int blocks = (int)std::min<size_t>((SN + 127) / 128, 152 * 8);
  k_shell_coef<<<blocks, 128, 0, st>>>(r, news, kperxkpar, del);
  ++*launches;
  return cudaPeekAtLastError() == cudaSuccess ? 0 : EPREM_GPU_ERR_CUDA;
}

template <typename Real>
static void shell_diffuse_as(const RunView &r, const int *ent, int L, const double *del,
                             void *out, int blocks, cudaStream_t st) {
  if (L <= 5)
    k_shell_diffuse<Real, 5><<<blocks, 256, 0, st>>>(r, ent, L, del, (Real *)out);
  else
    k_shell_diffuse<Real, 8><<<blocks, 256, 0, st>>>(r, ent, L, del, (Real *)out);
}

int launch_shell_diffuse(const RunView &r, const int *ent, int L, const double *del, void *out,
                         cudaStream_t st, uint64_t *launches) {
  const size_t total = (size_t)r.N * r.E * r.S * r.M;
  const int blocks = (int)std::min<size_t>((total + 511) / 512, 152 * 8);
  if (r.precision == EPREM_FP32)
    shell_diffuse_as<float>(r, ent, L, del, out, blocks, st);
  else
    shell_diffuse_as<double>(r, ent, L, del, out, blocks, st);
  ++*launches;
  return cudaPeekAtLastError() == cudaSuccess ? 0 : EPREM_GPU_ERR_CUDA;
}

}  // namespace eprem
