// stream3.cu -- streaming in the FP32 form, the two mu halves of a node on
// two lanes.
//
// DiffuseStreamData (src/energeticParticles.c:2240-2490), the upwind step in s
// with the BGK relaxation, as stream.cu / stream2.cu compute it, laid out so a
// thread holds half the registers of stream2.cu and twice as many warps fit
// on an SM:
//   * a warp holds 16 groups of NPT consecutive list nodes; lane g (0..15)
//     keeps the mu < 0 cells of group g, lane 16 + g its mu >= 0 cells;
//   * the mu >= 0 lanes store their nodes in reverse list order and the
//     negated multiplier, so both halves run the same instruction stream:
//       f[q] += (mult[q] del) (f[q] - f[q+1]),
//     whose last term takes its neighbour from lane +1 (mu < 0, the next
//     group's first node) or lane -1 (mu >= 0, the previous group's last
//     node) with one indexed shuffle; lanes 15 and 16 read theirs from the
//     warp halo, written by lane 0 / lane 31 of the neighbouring warps (and,
//     across CTAs of a cluster, into the neighbour CTA's shared memory);
//   * the relaxation mean adds the two halves with one xor-16 shuffle per
//     node.
// Per cell and sub-cycle the arithmetic is that of stream2.cu (products and
// fused multiply-adds in the same order); only the mean is summed as two
// half sums.
#include <cooperative_groups.h>

#include "common.cuh"
#include "kernels.h"

namespace cg = cooperative_groups;

namespace eprem {

// Threads per CTA and list nodes per thread, two shapes per mu bin (both
// spill-free): 0 fills the SM with 16 warps, 1 gives each thread more nodes
// (fewer shuffles per cell) at 12 warps.  A CTA holds NPT * T / 2 nodes.
template <int MMAX, int ALT> struct Stream3Shape;
template <> struct Stream3Shape<8, 0> { static constexpr int T = 512, NPT = 4; };
template <> struct Stream3Shape<16, 0> { static constexpr int T = 512, NPT = 4; };
template <> struct Stream3Shape<24, 0> { static constexpr int T = 512, NPT = 4; };
template <> struct Stream3Shape<32, 0> { static constexpr int T = 512, NPT = 4; };
template <> struct Stream3Shape<40, 0> { static constexpr int T = 512, NPT = 3; };
template <> struct Stream3Shape<48, 0> { static constexpr int T = 512, NPT = 2; };
template <> struct Stream3Shape<64, 0> { static constexpr int T = 512, NPT = 2; };
template <> struct Stream3Shape<8, 1> { static constexpr int T = 384, NPT = 6; };
template <> struct Stream3Shape<16, 1> { static constexpr int T = 384, NPT = 6; };
template <> struct Stream3Shape<24, 1> { static constexpr int T = 384, NPT = 5; };
template <> struct Stream3Shape<32, 1> { static constexpr int T = 384, NPT = 5; };
template <> struct Stream3Shape<40, 1> { static constexpr int T = 384, NPT = 4; };
template <> struct Stream3Shape<48, 1> { static constexpr int T = 384, NPT = 3; };
template <> struct Stream3Shape<64, 1> { static constexpr int T = 384, NPT = 2; };

template <int MMAX, int ALT>
constexpr size_t stream3_smem_bytes() {
  return sizeof(float) * 2 * 2 * (Stream3Shape<MMAX, ALT>::T / 32 + 1) * (MMAX / 2);
}

template <int MMAX, int ALT>
__global__ void __launch_bounds__((Stream3Shape<MMAX, ALT>::T), 1) k_stream3(RunView r, int m0) {
  constexpr int T = Stream3Shape<MMAX, ALT>::T;
  constexpr int NPT = Stream3Shape<MMAX, ALT>::NPT;
  constexpr int W = T / 32;
  constexpr int H = MMAX / 2;  // register slots of one half
  constexpr unsigned FULL = 0xffffffffu;
  extern __shared__ __align__(16) float halo[];  // [p][hi/lo][W+1][H]
  auto hi = [&](int p, int w) { return halo + ((p * 2 + 0) * (W + 1) + w) * H; };
  auto lo = [&](int p, int w) { return halo + ((p * 2 + 1) * (W + 1) + w) * H; };

  cg::cluster_group cluster = cg::this_cluster();
  const int C = (int)cluster.num_blocks();
  const int crank = (int)cluster.block_rank();
  const int s = blockIdx.y;
  const int e = r.E - 1 - (int)blockIdx.z;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int half = lane >> 4;  // 0: mu < 0 cells, 1: mu >= 0 cells
  const int M = r.M, N = r.N;
  const int nh = half ? M - m0 : m0;  // cells of this lane's half
  const int nmax = (M - m0) > m0 ? (M - m0) : m0;
  const int L = r.list_size[s];
  if (L < 3) return;

  const EnergyConsts ec = r.ec[e];
  const double dtMin = 0.4 * r.ds_min[s] * ec.vgrid_i;
  const double nst = floor(r.dt / dtMin + 1.0);
  if (!(nst <= (double)r.max_subcycles)) {
    if (crank == 0 && tid == 0) set_error(r.status, EPREM_GPU_ERR_SUBCYCLES, 1, s, -1, e, -1);
    return;
  }
  const int nsteps = (int)nst;
  const double dtProp = r.dt / (1.0 * nsteps);
  const double dtProp_i = 1.0 / dtProp;
  if (crank == 0 && tid == 0) {
    atomicMax(&r.status->max_stream, nsteps);
    atomicAdd(&r.status->stream_cs, (unsigned long long)nsteps * L * M);
  }
  for (int j = tid; j < 2 * 2 * (W + 1) * H; j += T) halo[j] = 0.f;

  // list index of this lane's node q: groups are NPT consecutive list nodes;
  // the mu >= 0 lanes hold theirs in reverse order
  const int group = (crank * T + warp * 32) / 2 + (lane & 15);
  const int i0 = NPT * group;
  auto list_index = [&](int q) { return half ? i0 + (NPT - 1 - q) : i0 + q; };
  const size_t sN = (size_t)s * N;
  const int cell0 = half ? m0 : 0;
  float F[NPT][H];
  // mult (negated on the mu >= 0 lanes; zero where the reference leaves the
  // half unchanged: the last list node for mu < 0, the first for mu >= 0),
  // relaxation factor exp(-dtProp/tau) and 1 - it, boundary seed
  float mult[NPT], em[NPT], om[NPT], bcv[NPT];
  __shared__ float s_bcv[3];  // seeds of list nodes 0..2 (the boundary)
  const double vdt = ec.vgrid * dtProp;
#pragma unroll
  for (int q = 0; q < NPT; ++q) {
    mult[q] = em[q] = om[q] = bcv[q] = 0.f;
    const int il = list_index(q);
    if (il < L) {
      const int k = r.list[sN + il];
      const size_t gidx = sN + k;
      const double tau = ec.vgrid_i * (ec.rig_lamo * r.mfp_node[gidx]);
      const double dsi = r.ds_i[sN + il];
      const double mu_ = (dtProp > tau) ? dsi * tau * dtProp_i : dsi * 1.0;
      const double emt = exp(-dtProp / tau);
      const bool edge = half ? (il == 0) : (il == L - 1);
      mult[q] = edge ? 0.f : (half ? -(float)mu_ : (float)mu_);
      em[q] = (float)emt;
      om[q] = (float)(1.0 - emt);
      bcv[q] = to_real<float>(seed_value(r, ec, r.seed_radial[gidx]));
      if (il < 3 && !half) s_bcv[il] = bcv[q];
    }
  }
  // f, floored at the seed when checkSeedPopulation is on: for a float v,
  // v < (float)seed selects the same cells as (double)v < seed, because no
  // float lies between seed and its rounding
#pragma unroll
  for (int q = 0; q < NPT; ++q) {
#pragma unroll
    for (int j = 0; j < H; ++j) F[q][j] = 0.f;
    const int il = list_index(q);
    if (il < L) {
      const size_t gidx = sN + r.list[sN + il];
      const float *fp = reinterpret_cast<const float *>(r.f) + (gidx * r.E + e) * M + cell0;
#pragma unroll
      for (int j = 0; j < H; ++j) {
        if (j < nh) {
          const float v = fp[j];
          F[q][j] = (r.check_seed && v < bcv[q]) ? bcv[q] : v;
        }
      }
    }
  }
  // del_fac(mu) = v dtProp mugrid(mu), mugrid(mu) = -1 + (mu + 1/2) dmu
  const float d0 =
      half ? (float)(vdt * r.mugrid[m0 < M ? m0 : M - 1]) : (float)(vdt * r.mugrid[0]);
  const float ddel = (float)(vdt * r.dmu);
  const float inv_m = (float)(1.0 / M);
  const int src = half ? lane - 1 : lane + 1;
  const bool from_halo = (lane == 15) || (lane == 16);
  float *next_hi0 = (C > 1 && crank < C - 1) ? cluster.map_shared_rank(halo, crank + 1) : nullptr;
  float *prev_loW = (C > 1 && crank > 0) ? cluster.map_shared_rank(halo, crank - 1) : nullptr;
  if (C > 1)
    cluster.sync();
  else
    __syncthreads();

  for (int step = 0; step < nsteps; ++step) {
    const int p = step & 1;
    if (r.use_bc && crank == 0 && warp == 0) {  // list nodes 0..2 live in warp 0
#pragma unroll
      for (int q = 0; q < NPT; ++q) {
        const int il = list_index(q);
        if (il < 3) {
          const float b = s_bcv[il];
#pragma unroll
          for (int j = 0; j < H; ++j) F[q][j] = b;
        }
      }
    }
    if (lane == 31) {  // last node's mu >= 0 half for the next warp's lane 16
      float *dst = hi(p, warp + 1);
      float *rdst = (warp == W - 1 && next_hi0) ? next_hi0 + ((p * 2 + 0) * (W + 1)) * H : nullptr;
#pragma unroll
      for (int j = 0; j < H; ++j)
        if (j < nh) {
          dst[j] = F[0][j];
          if (rdst) rdst[j] = F[0][j];
        }
    }
    if (lane == 0) {  // first node's mu < 0 half for the previous warp's lane 15
      float *dst = lo(p, warp);
      float *rdst = (warp == 0 && prev_loW) ? prev_loW + ((p * 2 + 1) * (W + 1) + W) * H : nullptr;
#pragma unroll
      for (int j = 0; j < H; ++j)
        if (j < nh) {
          dst[j] = F[0][j];
          if (rdst) rdst[j] = F[0][j];
        }
    }
    if (C > 1)
      cluster.sync();
    else
      __syncthreads();
    const float *edge = half ? hi(p, warp) : lo(p, warp + 1);
    float acc[NPT];
#pragma unroll
    for (int q = 0; q < NPT; ++q) acc[q] = 0.f;
#pragma unroll
    for (int j = 0; j < H; ++j) {
      if (j < nmax) {
        float del = d0 + (float)j * ddel;
        // opaque to loop-invariant code motion: otherwise the compiler hoists
        // every mult*del product out of the sub-cycle loop into registers
        asm volatile("" : "+f"(del));
        float nb = __shfl_sync(FULL, F[0][j], src);
        if (from_halo) nb = edge[j];
        if (j < nh) {
#pragma unroll
          for (int q = 0; q < NPT; ++q) {
            const float other = (q + 1 < NPT) ? F[q + 1 < NPT ? q + 1 : q][j] : nb;
            F[q][j] = F[q][j] + (mult[q] * del) * (F[q][j] - other);
            acc[q] += F[q][j];
          }
        }
      }
    }
#pragma unroll
    for (int q = 0; q < NPT; ++q) {
      const float tot = acc[q] + __shfl_xor_sync(FULL, acc[NPT - 1 - q], 16);
      const float iso = (inv_m * tot) * om[q];
#pragma unroll
      for (int j = 0; j < H; ++j)
        if (j < nmax) F[q][j] = F[q][j] * em[q] + iso;
    }
  }

#pragma unroll
  for (int q = 0; q < NPT; ++q) {
    const int il = list_index(q);
    if (il < L) {
      const int k = r.list[sN + il];
      int code = 0;
#pragma unroll
      for (int j = 0; j < H; ++j) {
        if (j < nh) {
          const float v = F[q][j];
          if (bad_value(v, &code)) set_error(r.status, code, 1, s, k, e, cell0 + j);
          F[q][j] = v < FLT_MIN ? FLT_MIN : v;
        }
      }
      // node k and the thinned nodes that reference it (previous list node + 1 .. k)
      const int kfirst = (il == 0) ? 0 : r.list[sN + il - 1] + 1;
      for (int kk = kfirst; kk <= k; ++kk) {
        float *op = reinterpret_cast<float *>(r.f) + ((sN + kk) * r.E + e) * M + cell0;
#pragma unroll
        for (int j = 0; j < H; ++j)
          if (j < nh) op[j] = F[q][j];
      }
    }
  }
  if (C > 1) cluster.sync();
}

template <int ALT>
static void shape_of(int mmax, int *T, int *npt) {
  switch (mmax) {
    case 8: *T = Stream3Shape<8, ALT>::T; *npt = Stream3Shape<8, ALT>::NPT; break;
    case 16: *T = Stream3Shape<16, ALT>::T; *npt = Stream3Shape<16, ALT>::NPT; break;
    case 24: *T = Stream3Shape<24, ALT>::T; *npt = Stream3Shape<24, ALT>::NPT; break;
    case 32: *T = Stream3Shape<32, ALT>::T; *npt = Stream3Shape<32, ALT>::NPT; break;
    case 40: *T = Stream3Shape<40, ALT>::T; *npt = Stream3Shape<40, ALT>::NPT; break;
    case 48: *T = Stream3Shape<48, ALT>::T; *npt = Stream3Shape<48, ALT>::NPT; break;
    default: *T = Stream3Shape<64, ALT>::T; *npt = Stream3Shape<64, ALT>::NPT; break;
  }
}

int plan_stream3(int N, int M, int m0, int alt, StreamPlan *plan) {
  int mmax = 0;
  for (int b : {8, 16, 24, 32, 40, 48, 64})
    if (M <= b && m0 <= b / 2 && M - m0 <= b / 2) { mmax = b; break; }
  if (!mmax) return EPREM_GPU_ERR_ARG;
  int T, npt;
  if (alt)
    shape_of<1>(mmax, &T, &npt);
  else
    shape_of<0>(mmax, &T, &npt);
  plan->mmax = mmax;
  plan->threads = T;
  plan->reg_coef = 3 + (alt ? 1 : 0);  // marks the split-halves kernel and its shape
  const int per_cta = npt * (T / 2);
  plan->cluster = (N + per_cta - 1) / per_cta;
  return plan->cluster > 8 ? EPREM_GPU_ERR_ARG : 0;
}

template <int MMAX, int ALT>
static cudaError_t launch_stream3_t(const RunView &r, int cluster, int m0, cudaStream_t st) {
  constexpr int T = Stream3Shape<MMAX, ALT>::T;
  constexpr size_t dyn = stream3_smem_bytes<MMAX, ALT>();
  auto kern = k_stream3<MMAX, ALT>;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(cluster, r.S, r.E);
  cfg.blockDim = dim3(T, 1, 1);
  cfg.dynamicSmemBytes = dyn;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = cluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, r, m0);
}

template <int ALT>
static cudaError_t launch_alt(const RunView &r, const StreamPlan &pl, int m0, cudaStream_t st) {
  switch (pl.mmax) {
    case 8: return launch_stream3_t<8, ALT>(r, pl.cluster, m0, st);
    case 16: return launch_stream3_t<16, ALT>(r, pl.cluster, m0, st);
    case 24: return launch_stream3_t<24, ALT>(r, pl.cluster, m0, st);
    case 32: return launch_stream3_t<32, ALT>(r, pl.cluster, m0, st);
    case 40: return launch_stream3_t<40, ALT>(r, pl.cluster, m0, st);
    case 48: return launch_stream3_t<48, ALT>(r, pl.cluster, m0, st);
    default: return launch_stream3_t<64, ALT>(r, pl.cluster, m0, st);
  }
}

int launch_stream3(const RunView &r, const StreamPlan &pl, int m0, cudaStream_t st,
                   uint64_t *launches) {
  const cudaError_t err =
      pl.reg_coef == 4 ? launch_alt<1>(r, pl, m0, st) : launch_alt<0>(r, pl, m0, st);
  *launches += 1;
  return err == cudaSuccess ? 0 : EPREM_GPU_ERR_CUDA;
}

}  // namespace eprem
