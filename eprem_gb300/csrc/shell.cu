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
// the four fractions and their sum, del[((s*N + k)*E + e)*5 + {0..3, 4}].
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
      double *out = del + (g * r.E + e) * 5;
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

// One thread per cell of nodes 1..N-1, ordered (k, e, stream, mu): one
// (node, energy) slice of all streams is in flight at a time, so the
// neighbours' reads of a slice come from L2.  Writes f + delta to out (same
// layout as f); the caller copies it back once every cell has been read.
// ent[p] = source stream * 8 + direction (0..3 north..south, 4 own loss).
template <typename Real>
__global__ void k_shell_diffuse(RunView r, const int *rowptr, const int *ent, const double *del,
                                Real *out) {
  const Real *f = static_cast<const Real *>(r.f);
  const size_t M = r.M, S = r.S, E = r.E;
  const size_t per_stream = (size_t)r.N * E * M;
  const size_t total = (size_t)(r.N - 1) * E * S * M;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const int m = (int)(t % M);
    size_t q = t / M;
    const int s = (int)(q % S);
    q /= S;
    const int e = (int)(q % E);
    const int k = 1 + (int)(q / E);
    const size_t off = ((size_t)k * E + e) * M + m;
    const size_t ke5 = ((size_t)k * E + e) * 5;
    Real acc = Real(0);
    const int p1 = rowptr[s + 1];
    for (int p = rowptr[s]; p < p1; p++) {
      const int code = ent[p];
      const int i = code >> 3, d = code & 7;
      const Real a = (Real)del[(size_t)i * r.N * E * 5 + ke5 + d];
      const Real fi = f[(size_t)i * per_stream + off];
      acc = d < 4 ? sd_fma(a, fi, acc) : sd_fms(a, fi, acc);
    }
    const size_t gi = (size_t)s * per_stream + off;
    const Real v = f[gi] + acc;
    out[gi] = v;
    if (isnan((double)v) || isinf((double)v))
      set_error(r, isnan((double)v) ? EPREM_GPU_ERR_NAN : EPREM_GPU_ERR_INF, 6, s, k, e, m);
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

int launch_shell_diffuse(const RunView &r, const int *rowptr, const int *ent, const double *del,
                         void *scratch, cudaStream_t st, uint64_t *launches) {
  const size_t total = (size_t)(r.N - 1) * r.E * r.S * r.M;
  const int blocks = (int)std::min<size_t>((total + 255) / 256, 152 * 16);
  if (r.precision == EPREM_FP32)
    k_shell_diffuse<float><<<blocks, 256, 0, st>>>(r, rowptr, ent, del, (float *)scratch);
  else
    k_shell_diffuse<double><<<blocks, 256, 0, st>>>(r, rowptr, ent, del, (double *)scratch);
  ++*launches;
  if (cudaPeekAtLastError() != cudaSuccess) return EPREM_GPU_ERR_CUDA;
  // nodes 1..N-1 of every stream back into f
  const size_t elem = r.precision == EPREM_FP32 ? sizeof(float) : sizeof(double);
  const size_t em = (size_t)r.E * r.M, pitch = (size_t)r.N * em * elem;
  char *dst = static_cast<char *>(r.f) + em * elem;
  const char *src = static_cast<const char *>(scratch) + em * elem;
  return cudaMemcpy2DAsync(dst, pitch, src, pitch, (size_t)(r.N - 1) * em * elem, r.S,
                           cudaMemcpyDeviceToDevice, st) == cudaSuccess
             ? 0
             : EPREM_GPU_ERR_CUDA;
}

}  // namespace eprem
