// node32.cu -- focusing and adiabatic change per node in the FP32 form (K23').
//
// Same operators as node.cu (AdiabaticFocusing src/energeticParticles.c:
// 1537-1803, AdiabaticChange :808-1077, Euler upwind operators :1084-1176,
// :1809-1895), arranged for the FP32 pipe:
//   * each thread owns one (node, energy) row for focusing and one (node, mu)
//     column for the change, with the cells *and* the pre-scaled face
//     velocities of its line in registers -- no shared-memory traffic inside
//     the sub-cycle loops;
//   * the CFL maxima stay FP64 (as the form requires) but are taken where they
//     lie: focusing's face velocity 1/4 (1-mu^2)(a_E + mu b) summed over two
//     cells is linear in a_E, so its maximum over energies is on the rows of
//     the smallest and largest a_E; the change velocity cool (a_mu/v + b_mu)
//     is linear in 1/v, which is monotonic in energy, so its maximum is on the
//     first and last energy rows.  The rows are evaluated with the reference's
//     expressions, without fused multiply-adds.
// Only the Euler upwind algorithm (alg 1) runs here; RK3 / WENO3 use node.cu.
#include "common.cuh"
#include "kernels.h"

namespace eprem {

constexpr int kNode32Threads = 128;
constexpr int kNode32MaxNodes = 16;

__device__ __forceinline__ double m_(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double a_(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double s_(double a, double b) { return __dsub_rn(a, b); }

template <int P>
__global__ void __launch_bounds__(kNode32Threads) k_node32(RunView r, int G) {
  extern __shared__ __align__(16) float slab[];  // [G][E][M]
  __shared__ double n_dupar[kNode32MaxNodes], n_b[kNode32MaxNodes], n_dlnbds[kNode32MaxNodes];
  __shared__ double n_cool[kNode32MaxNodes], n_dlnbdt[kNode32MaxNodes], n_dlnndt[kNode32MaxNodes];
  __shared__ float n_scale_f[kNode32MaxNodes], n_scale_c[kNode32MaxNodes];
  __shared__ float n_bc0[kNode32MaxNodes], n_bc1[kNode32MaxNodes];
  __shared__ int n_sub_f[kNode32MaxNodes], n_sub_c[kNode32MaxNodes], n_ok[kNode32MaxNodes];
  __shared__ float s_mu[64], s_vi[64];
  const int E = r.E, M = r.M, N = r.N, EM = E * M;
  const int tid = threadIdx.x;
  const size_t SN = (size_t)r.S * N;
  const size_t g0 = (size_t)blockIdx.x * G;
  const int Gv = (int)((SN - g0) < (size_t)G ? (SN - g0) : (size_t)G);
  float *fg = reinterpret_cast<float *>(r.f) + g0 * EM;
  for (int i = tid; i < Gv * EM; i += kNode32Threads) slab[i] = fg[i];
  if (tid < M) s_mu[tid] = (float)r.mugrid[tid];
  if (tid < E) s_vi[tid] = (float)r.ec[tid].vgrid_i;
  const double dt = r.dt, dt_full = r.dt_full;

  // ---- per-node scalars, FP64 CFL from the extreme rows --------------------
  if (tid < Gv) {
    const size_t g = g0 + tid;
    const bool ok = (g % N) != 0;  // node 0 is the spawn node (innerComputeShell)
    n_ok[tid] = ok;
    const double dupar = node_field(r, EPREM_NODE_DUPAR)[g] / dt_full;
    const double dlnb = node_field(r, EPREM_NODE_DLNB)[g] / dt_full;
    const double dlnn = node_field(r, EPREM_NODE_DLNN)[g] / dt_full;
    int ns_f = 0, ns_c = 0;
    if (r.use_focus) {
      const double b = s_(m_(2.0, dlnn), m_(3.0, dlnb));
      const double bp = node_field(r, EPREM_NODE_BMAG_PLUS)[g];
      const double bm = node_field(r, EPREM_NODE_BMAG_MINUS)[g];
      const double dlnbds = (bp == 0.0 || bm == 0.0)
                                ? 0.0
                                : (log(bp) - log(bm)) / a_(m_(2.0, node_field(r, EPREM_NODE_DS)[g]), DBL_MIN);
      double amin = 0.0, amax = 0.0;
      for (int e = 0; e < E; e++) {
        const double v = r.ec[e].vgrid;
        const double a = s_(m_(-v, dlnbds), m_(2.0 / v, dupar));
        if (e == 0 || a < amin) amin = a;
        if (e == 0 || a > amax) amax = a;
      }
      double vmax = 0.0;
      for (int pass = 0; pass < 2; pass++) {
        const double a = pass ? amax : amin;
        double vel_prev = 0.0;
        for (int m = 0; m < M; m++) {
          const double mu = r.mugrid[m];
          const double vel = m_(m_(0.5, s_(1.0, m_(mu, mu))), a_(a, m_(mu, b)));
          if (m >= 1) vmax = fmax(vmax, fabs(m_(0.5, a_(vel, vel_prev))));
          vel_prev = vel;
        }
      }
      const double nsub = ceil(dt / (m_(0.9, r.dmu) / vmax));
      if (!(nsub <= (double)r.max_subcycles)) {
        if (ok) set_error(r.status, EPREM_GPU_ERR_SUBCYCLES, 2, (int)(g / N), (int)(g % N), -1, -1);
      } else {
        ns_f = (int)nsub;
      }
      if (!ok) ns_f = 0;
      n_dupar[tid] = dupar;
      n_b[tid] = b;
      n_dlnbds[tid] = dlnbds;
      n_scale_f[tid] = (float)((dt / ns_f) / r.dmu);
    }
    if (r.use_change) {
      const double cool = (dlnn < 0) ? 1.0 - r.damp_cooling : 1.0;
      double vmax = 0.0;
      for (int pass = 0; pass < 2; pass++) {
        const double vi = r.ec[pass ? E - 1 : 0].vgrid_i;
        for (int m = 0; m < M; m++) {
          const double mu = r.mugrid[m];
          const double a = m_(-mu, dupar);
          const double bb = a_(m_(m_(mu, mu), s_(dlnn, dlnb)), m_(m_(0.5, s_(1.0, m_(mu, mu))), dlnb));
          vmax = fmax(vmax, fabs(m_(cool, a_(m_(a, vi), bb))));
        }
      }
      const double nsub = ceil(dt / (m_(0.9, r.dlnp) / vmax));
      if (!(nsub <= (double)r.max_subcycles)) {
        if (ok) set_error(r.status, EPREM_GPU_ERR_SUBCYCLES, 3, (int)(g / N), (int)(g % N), -1, -1);
      } else {
        ns_c = (int)nsub;
      }
      if (!ok) ns_c = 0;
      n_cool[tid] = cool;
      n_dlnbdt[tid] = dlnb;
      n_dlnndt[tid] = dlnn;
      n_scale_c[tid] = (float)((dt / ns_c) / r.dlnp);
      const double radial = r.seed_radial[g];
      n_bc0[tid] = (float)log(seed_value(r, r.ec[0], radial));
      n_bc1[tid] = (float)log(seed_value(r, r.ec[E - 1], radial));
    }
    n_sub_f[tid] = ns_f;
    n_sub_c[tid] = ns_c;
    if (ok) {
      atomicMax(&r.status->max_focus, ns_f);
      atomicMax(&r.status->max_change, ns_c);
      atomicAdd(&r.status->focus_cs, (unsigned long long)ns_f * EM);
      atomicAdd(&r.status->change_cs, (unsigned long long)ns_c * EM);
    }
  }
  __syncthreads();

  // ---- focusing: one energy row per thread --------------------------------
  if (r.use_focus) {
    for (int it = tid; it < Gv * E; it += kNode32Threads) {
      const int g = it / E, e = it % E;
      if (!n_ok[g]) continue;
      float *row = slab + (size_t)g * EM + e * M;
      const int ns = n_sub_f[g];
      float fr[P];
#pragma unroll
      for (int m = 0; m < P; ++m)
        if (m < M) fr[m] = row[m];
      if (ns > 0) {
        const double v = r.ec[e].vgrid;
        const float a = (float)(-v * n_dlnbds[g] - (2.0 / v) * n_dupar[g]);
        const float b = (float)n_b[g];
        const float sc = n_scale_f[g];
        // q[j] = dt_sub/dmu * (vel(mu_{j-1}) + vel(mu_j))/2, interior faces 1..M-1
        float q[P + 1];
        float vel_prev = 0.f;
#pragma unroll
        for (int m = 0; m < P; ++m) {
          if (m < M) {
            const float mu = s_mu[m];
            const float vel = 0.5f * (1.f - mu * mu) * (a + mu * b);
            if (m >= 1) q[m] = sc * 0.5f * (vel + vel_prev);
            vel_prev = vel;
          }
        }
        for (int s = 0; s < ns; ++s) {
          float gprev = 0.f;
#pragma unroll
          for (int m = 0; m < P; ++m) {
            if (m < M) {
              float gnext = 0.f;
              if (m + 1 < M) {
                const float qq = q[m + 1];
                gnext = qq * (qq >= 0.f ? fr[m] : fr[m + 1]);
              }
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
          if (bad_value(v, &code)) {
            const size_t gg = g0 + g;
            set_error(r.status, code, 2, (int)(gg / N), (int)(gg % N), e, m);
          }
          row[m] = v < FLT_MIN ? FLT_MIN : v;
        }
      }
    }
    __syncthreads();
  }

  // ---- adiabatic change: one mu column per thread --------------------------
  if (r.use_change) {
    for (int it = tid; it < Gv * M; it += kNode32Threads) {
      const int g = it / M, m = it % M;
      if (!n_ok[g]) continue;
      float *col = slab + (size_t)g * EM + m;  // stride M
      const int ns = n_sub_c[g];
      float fc[P];
#pragma unroll
      for (int e = 0; e < P; ++e)
        if (e < E) fc[e] = logf(col[e * M]);
      if (ns > 0) {
        const double mu = r.mugrid[m];
        const float am = (float)(-mu * n_dupar[g]);
        const float bm = (float)(mu * mu * (n_dlnndt[g] - n_dlnbdt[g]) +
                                 0.5 * (1.0 - mu * mu) * n_dlnbdt[g]);
        const float cool = (float)n_cool[g];
        const float sc = n_scale_c[g];
        const float bc0 = n_bc0[g], bc1 = n_bc1[g];
        float q[P + 1];
        float vel_prev = 0.f;
#pragma unroll
        for (int e = 0; e < P; ++e) {
          if (e < E) {
            const float vel = cool * (am * s_vi[e] + bm);
            if (e >= 1) q[e] = sc * 0.5f * (vel + vel_prev);
            vel_prev = vel;
          }
        }
        for (int s = 0; s < ns; ++s) {
          const float q1 = q[1];
          float gprev = q1 * (q1 >= 0.f ? fc[0] : fc[1]);
          const float d0 = (q1 <= 0.f) ? q1 * (fc[1] - fc[0]) : q1 * (fc[0] - bc0);
          float fold_prev = fc[0];
          fc[0] = fc[0] - d0;
#pragma unroll
          for (int e = 1; e < P; ++e) {
            if (e < E - 1) {
              const float qq = q[e + 1];
              const float gnext = qq * (qq >= 0.f ? fc[e] : fc[e + 1]);
              fold_prev = fc[e];
              fc[e] = fc[e] - (gnext - gprev);
              gprev = gnext;
            } else if (e == E - 1) {
              const float qq = q[E - 1];
              const float dl = (qq >= 0.f) ? qq * (fc[e] - fold_prev) : qq * (bc1 - fc[e]);
              fc[e] = fc[e] - dl;
            }
          }
        }
      }
      int code = 0;
#pragma unroll
      for (int e = 0; e < P; ++e) {
        if (e < E) {
          const float v = expf(fc[e]);
          if (bad_value(v, &code)) {
            const size_t gg = g0 + g;
            set_error(r.status, code, 3, (int)(gg / N), (int)(gg % N), e, m);
          }
          col[e * M] = v < FLT_MIN ? FLT_MIN : v;
        }
      }
    }
    __syncthreads();
  }
  for (int i = tid; i < Gv * EM; i += kNode32Threads) fg[i] = slab[i];
}

int plan_node32(int E, int M, NodePlan *plan) {
  const int mx = E > M ? E : M;
  int p = 0;
  for (int b : {8, 16, 24, 32, 48, 64})
    if (mx <= b) { p = b; break; }
  if (!p || E > 64 || M > 64) return EPREM_GPU_ERR_ARG;
  plan->pmax = p;
  plan->threads = kNode32Threads;
  const size_t per = (size_t)E * M * sizeof(float);
  int G = (int)((48 * 1024) / per);
  if (G > kNode32MaxNodes) G = kNode32MaxNodes;
  if (G < 1) G = 1;
  plan->nodes = G;
  plan->smem = per * G;
  return plan->smem > 200 * 1024 ? EPREM_GPU_ERR_ARG : 0;
}

template <int P>
static cudaError_t launch_node32_t(const RunView &r, const NodePlan &pl, cudaStream_t st) {
  auto kern = k_node32<P>;
  cudaError_t err =
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pl.smem);
  if (err != cudaSuccess) return err;
  const size_t SN = (size_t)r.S * r.N;
  const unsigned blocks = (unsigned)((SN + pl.nodes - 1) / pl.nodes);
  kern<<<blocks, kNode32Threads, pl.smem, st>>>(r, pl.nodes);
  return cudaGetLastError();
}

int launch_node32(const RunView &r, const NodePlan &pl, cudaStream_t st, uint64_t *launches) {
  cudaError_t err;
  switch (pl.pmax) {
    case 8: err = launch_node32_t<8>(r, pl, st); break;
    case 16: err = launch_node32_t<16>(r, pl, st); break;
    case 24: err = launch_node32_t<24>(r, pl, st); break;
    case 32: err = launch_node32_t<32>(r, pl, st); break;
    case 48: err = launch_node32_t<48>(r, pl, st); break;
    default: err = launch_node32_t<64>(r, pl, st); break;
  }
  *launches += 1;
  return err == cudaSuccess ? 0 : EPREM_GPU_ERR_CUDA;
}

}  // namespace eprem
