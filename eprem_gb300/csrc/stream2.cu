// stream2.cu -- streaming in the FP32 form with several list nodes per thread.
//
// DiffuseStreamData (src/energeticParticles.c:2240-2490) as in stream.cu, but
// shaped for the FP32 pipe, where the per-cell cost of shuffles and shared-
// memory loads, not arithmetic, limited the one-node-per-thread kernel:
//   * thread i owns NPT consecutive list nodes; inside the thread a node's
//     upwind neighbour is the next register array, across threads one shuffle
//     serves NPT cells;
//   * the upwind coefficient mult*del_fac is formed per cell from the node's
//     mult (register) and del_fac(mu) = v dtProp mugrid(mu), evaluated from
//     the uniform mu grid (mugrid = -1 + (mu + 1/2) dmu) -- no per-cell load;
//   * a thread keeps each node's cells in two register halves, mu < 0 and
//     mu >= 0 (the mu grid is increasing, so the split is one index m0); each
//     half has its own loop, so the upwind direction is never a branch;
//   * warp-edge lanes publish only the half their neighbour needs (lane 31's
//     last node for mu >= 0, lane 0's first node for mu < 0).
// A CTA of T threads holds NPT*T list nodes (shapes per mu bin below; a
// 1000-node stream fits one CTA of the default shapes).  Three kernels: k_stream2, the scalar
// shape (any M and split), k_stream2_pairs, the packed fp32x2 shapes, with f
// held as float2 pairs (an odd half padded with a zero cell), and
// k_stream2_mirror, the packed shape with the mu < 0 half in mirror order so
// that one upwind coefficient serves a cell of each half (coefficients in
// shared memory; on one CTA per slab, warps hand their halo rows to their
// neighbours through mbarriers instead of a CTA barrier per sub-cycle).
#include <cooperative_groups.h>

#include "common.cuh"
#include "kernels.h"

namespace cg = cooperative_groups;

namespace eprem {

// CTA shapes (threads T, list nodes per thread NPT) per mu bin, the bin's
// default first.  A thread holds NPT nodes x MMAX cells in registers: NPT * T
// list nodes per CTA, clusters of CTAs for longer streams.  Fewer nodes per
// thread leave registers for more warps per SM; more nodes per thread amortise
// the shuffles and halo exchange over more cells.  plan_stream2 picks a shape
// from N (or the one a variant names), the autotuner times them all.
// Measured on a GB300 (96 streams x 50 E x 40 mu, FP32 FMA-peak fractions of
// the compile-time-guard kernel): N = 1000 -- 256x4 0.42, 128x4 in clusters
// of 2 0.40, 256x3 in clusters of 2 0.24, 384x3 and 512x2 (register spills)
// 0.24; N = 1500 -- 128x4 in clusters of 3 0.39, 256x3 in clusters of 2
// 0.37, 384x2 in clusters of 2 (12 warps/SM, 168 registers) 0.34, 256x4 in
// clusters of 2 (27 % of the slots idle) 0.29.  More warps per SM at fewer
// registers lost at both sizes: 352x3 and 512x2 (register-capped, spilling)
// 0.24 at N = 1000.  Shapes that spill are not kept; where two shapes waste
// as few slots, the earlier wins.
#define EPREM_S2_SHAPES(X)                                                             \
  X(8, 512, 2) X(16, 512, 2) X(24, 512, 2) X(24, 256, 4) X(24, 128, 4) X(32, 256, 4)  \
  X(32, 128, 4) X(32, 256, 3) X(40, 256, 4) X(40, 128, 4) X(40, 256, 3) X(48, 256, 3) \
  X(48, 128, 3) X(64, 256, 2) X(64, 128, 2)

// The relaxation weight of one sub-cycle, f <- f (1 - om) + iso om with
// om = 1 - exp(-dtProp/tau).  For the sum over mu to be kept, 1 - om must be
// exact in float, so om is a multiple of 2^-24; rounding it there once moved
// the relaxation rate by up to 2^-25 / om (1e-4 at the 1536-stream case,
// whose om is 3e-4 - 1e-3), a bias that the diffusive tail of the
// distribution turns into 1e-3 of the flux 15 decades below its peak.  So
// om alternates between the two multiples around it (omlo and omlo +
// 2^-24) with an error-diffusion counter: over any run of sub-cycles the
// weights sum to the exact om times their number within 2^-24, and every
// single sub-cycle still keeps the sum.  Splitting the weight apart, f +
// om (iso - f), would do the same at one more packed operation per cell
// pair.  dith starts at 1/2 in every launch; phi is om 2^24 - omlo 2^24.
__device__ __forceinline__ float relax_weight(float omlo, float phi, float &dith) {
  dith += phi;
  const bool up = dith >= 1.f;
  dith = up ? dith - 1.f : dith;
  return up ? omlo + 0x1p-24f : omlo;
}

// The common exponent of a (stream, energy) slab (FP32 row exponents): the
// largest true value of its rows, and of the seeds the sub-step can write,
// brought to [2^kRowTop, 2^(kRowTop+1)).  lg: this thread's largest
// floor(log2) of a true value; red: W + 1 ints of shared memory.  A cluster's
// CTAs combine their maxima through distributed shared memory (the slot read
// remotely is written once per launch, and the kernel ends in a cluster
// barrier, so no CTA leaves while it is read).
template <int T>
__device__ __forceinline__ int slab_exp(int lg, int *red, cg::cluster_group &cluster, int C) {
  constexpr int W = T / 32;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  lg = __reduce_max_sync(0xffffffffu, lg);
  if (lane == 0) red[warp] = lg;
  __syncthreads();
  if (threadIdx.x == 0) {
    int m = red[0];
    for (int w = 1; w < W; ++w) m = max(m, red[w]);
    red[W] = m;
  }
  if (C > 1)
    cluster.sync();
  else
    __syncthreads();
  int m = red[W];
  for (int c = 0; c < C && C > 1; ++c) m = max(m, cluster.map_shared_rank(red, c)[W]);
  return row_exp_for(m);
}

// The two power-of-two factors of ldexp_f(x, k), formed once for a row.
struct Pow2Pair {
  float a, b;
};
__device__ __forceinline__ Pow2Pair pow2_pair(int k) {
  const int k1 = k > 127 ? 127 : (k < -126 ? -126 : k);
  int k2 = k - k1;
  k2 = k2 > 127 ? 127 : (k2 < -126 ? -126 : k2);
  return Pow2Pair{pow2f(k1), pow2f(k2)};
}
__device__ __forceinline__ float scale2(float x, Pow2Pair p) { return (x * p.a) * p.b; }

template <int MMAX, int T>
constexpr size_t stream2_smem_bytes() {
  return sizeof(float) * 2 * 2 * (T / 32 + 1) * (MMAX / 2);
}

// The scalar shape: any M up to MMAX and any split m0 (odd halves included).
template <int MMAX, int T, int NPT>
__global__ void __launch_bounds__(T, 1) k_stream2(RunView r, int m0) {
  constexpr int W = T / 32;
  constexpr int H = MMAX / 2;  // register slots per direction (mu < 0, mu >= 0)
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
  const int M = r.M, N = r.N;
  // cells moving toward the inner / outer end
  const int nL = m0, nR = M - m0;
  const int L = r.list_size[s];
  if (L < 3) return;

  const EnergyConsts ec = r.ec[e];
  const double dtMin = 0.4 * r.ds_min[s] * ec.vgrid_i;
  const double nst = floor(r.dt / dtMin + 1.0);
  if (!(nst <= (double)r.max_subcycles)) {
    if (crank == 0 && tid == 0) set_error(r, EPREM_GPU_ERR_SUBCYCLES, 1, s, -1, e, -1);
    return;
  }
  const int nsteps = (int)nst;
  const double dtProp = r.dt / (1.0 * nsteps);
  if (crank == 0 && tid == 0) {
    atomicMax(&r.status->max_stream, nsteps);
    atomicAdd(&r.status->stream_cs, (unsigned long long)nsteps * L * M);
  }
  for (int j = tid; j < 2 * 2 * (W + 1) * H; j += T) halo[j] = 0.f;

  const int i0 = NPT * (crank * T + tid);  // list index of this thread's first node
  const size_t sN = (size_t)s * N;
  // Lf[q] holds node q's mu = j cells (mu < 0), Rf[q] its mu = m0 + j cells
  float Lf[NPT][H], Rf[NPT][H];
  // per node: mult for each upwind direction (zero where the reference leaves
  // the cell unchanged: first list node for mu >= 0, last for mu < 0),
  // relaxation factor exp(-dtProp/tau) and 1 - it, boundary seed
  float mhi[NPT], mlo[NPT], phi[NPT], omlo[NPT], dith[NPT];
  __shared__ float s_bcv[3];  // seeds of list nodes 0..2, the boundary (CTA rank 0)
  __shared__ int s_red[W + 1];
  const double vdt = ec.vgrid * dtProp;
  // per list node: mult, relaxation factor and its complement, seed * 2^seed_k,
  // made in FP64 once per call (k_stream2_coef) and rounded to float
  const float4 *cf = r.scoef + ((size_t)s * r.E + e) * N;
  int xr[NPT];      // the rows' exponents as loaded
  float sw[NPT];    // seed * 2^seed_k
  int lg = kNoExp;  // largest floor(log2) of a true value of this thread's rows and seeds
  const bool seeds_in = r.check_seed != 0;
#pragma unroll
  for (int q = 0; q < NPT; ++q) {
    mhi[q] = mlo[q] = phi[q] = omlo[q] = 0.f;
    dith[q] = 0.5f;
    xr[q] = 0;
    sw[q] = 0.f;
#pragma unroll
    for (int j = 0; j < H; ++j) Lf[q][j] = Rf[q][j] = 0.f;
    const int il = i0 + q;
    if (il < L) {
      const int k = r.list[sN + il];
      const size_t gidx = sN + k;
      const float4 c = cf[il];
      const float *fp = reinterpret_cast<const float *>(r.f) + (gidx * r.E + e) * M;
      float mx = 0.f;
#pragma unroll
      for (int j = 0; j < H; ++j) {
        if (j < nL) {
          Lf[q][j] = fp[j];
          mx = fmaxf(mx, Lf[q][j]);
        }
        if (j < nR) {
          Rf[q][j] = fp[m0 + j];
          mx = fmaxf(mx, Rf[q][j]);
        }
      }
      xr[q] = r.fexp[gidx * r.E + e];
      sw[q] = c.w;
      const int lr = ilogb_f(mx);
      if (lr != kNoExp) lg = max(lg, lr - xr[q]);
      const int ls = ilogb_f(c.w);
      if ((seeds_in || (r.use_bc && il < 3)) && ls != kNoExp) lg = max(lg, ls - ec.seed_k);
      mhi[q] = (il == 0) ? 0.f : c.x;
      mlo[q] = (il == L - 1) ? 0.f : c.x;
      phi[q] = c.y;
      omlo[q] = c.z;
    }
  }
  // the slab's common exponent; rows and seeds brought to it (exact powers of two)
  const int K = slab_exp<T>(lg, s_red, cluster, C);
#pragma unroll
  for (int q = 0; q < NPT; ++q) {
    const int il = i0 + q;
    if (il < L) {
      const Pow2Pair pf = pow2_pair(K - xr[q]);
      const float seedf = scale2(sw[q], pow2_pair(K - ec.seed_k));
#pragma unroll
      for (int j = 0; j < H; ++j) {
        if (j < nL) {
          float v = scale2(Lf[q][j], pf);
          if (seeds_in && v < seedf) v = seedf;  // seedPopulationCheck
          Lf[q][j] = v;
        }
        if (j < nR) {
          float v = scale2(Rf[q][j], pf);
          if (seeds_in && v < seedf) v = seedf;
          Rf[q][j] = v;
        }
      }
      if (il < 3) s_bcv[il] = seedf;
    }
  }
  // del_fac(mu) = v dtProp mugrid(mu), mugrid(mu) = -1 + (mu + 1/2) dmu
  const float dl0 = (float)(vdt * r.mugrid[0]);
  const float dr0 = (float)(vdt * r.mugrid[m0 < M ? m0 : M - 1]);
  const float ddel = (float)(vdt * r.dmu);
  const float inv_m = (float)(1.0 / M);
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
        const int il = i0 + q;
        if (il < 3) {
          const float b = s_bcv[il];
#pragma unroll
          for (int j = 0; j < H; ++j) Lf[q][j] = Rf[q][j] = b;
        }
      }
    }
    if (lane == 31) {  // last node's outward half for the next warp's first node
      float *dst = hi(p, warp + 1);
      float *rdst = (warp == W - 1 && next_hi0) ? next_hi0 + ((p * 2 + 0) * (W + 1)) * H : nullptr;
#pragma unroll
      for (int j = 0; j < H; ++j)
        if (j < nR) {
          dst[j] = Rf[NPT - 1][j];
          if (rdst) rdst[j] = Rf[NPT - 1][j];
        }
    }
    if (lane == 0) {  // first node's inward half for the previous warp's last node
      float *dst = lo(p, warp);
      float *rdst = (warp == 0 && prev_loW) ? prev_loW + ((p * 2 + 1) * (W + 1) + W) * H : nullptr;
#pragma unroll
      for (int j = 0; j < H; ++j)
        if (j < nL) {
          dst[j] = Lf[0][j];
          if (rdst) rdst[j] = Lf[0][j];
        }
    }
    if (C > 1)
      cluster.sync();
    else
      __syncthreads();
    const float *my_hi = hi(p, warp);
    const float *my_lo = lo(p, warp + 1);
    float acc[NPT];
#pragma unroll
    for (int q = 0; q < NPT; ++q) acc[q] = 0.f;
    // mu < 0: upwind from the outer neighbour (list node + 1), old values
#pragma unroll
    for (int j = 0; j < H; ++j) {
      if (j < nL) {
        float del = dl0 + (float)j * ddel;
        // opaque to loop-invariant code motion: otherwise the compiler hoists
        // every mult*del product out of the sub-cycle loop into registers
        asm volatile("" : "+f"(del));
        float nb = __shfl_down_sync(FULL, Lf[0][j], 1);
        if (lane == 31) nb = my_lo[j];
#pragma unroll
        for (int q = 0; q < NPT; ++q) {
          const float right = (q + 1 < NPT) ? Lf[q + 1 < NPT ? q + 1 : q][j] : nb;
          Lf[q][j] = Lf[q][j] + (mlo[q] * del) * (Lf[q][j] - right);
          acc[q] += Lf[q][j];
        }
      }
    }
    // mu >= 0: upwind from the inner neighbour (list node - 1), old values
#pragma unroll
    for (int j = 0; j < H; ++j) {
      if (j < nR) {
        float del = dr0 + (float)j * ddel;
        asm volatile("" : "+f"(del));
        float nb = __shfl_up_sync(FULL, Rf[NPT - 1][j], 1);
        if (lane == 0) nb = my_hi[j];
#pragma unroll
        for (int q = NPT - 1; q >= 0; --q) {
          const float left = (q > 0) ? Rf[q > 0 ? q - 1 : 0][j] : nb;
          Rf[q][j] = Rf[q][j] + (mhi[q] * del) * (left - Rf[q][j]);
          acc[q] += Rf[q][j];
        }
      }
    }
#pragma unroll
    for (int q = 0; q < NPT; ++q) {
      const float om = relax_weight(omlo[q], phi[q], dith[q]), em = 1.f - om;
      const float iso = (inv_m * acc[q]) * om;
#pragma unroll
      for (int j = 0; j < H; ++j) {
        Lf[q][j] = Lf[q][j] * em + iso;
        Rf[q][j] = Rf[q][j] * em + iso;
      }
    }
  }

#pragma unroll
  for (int q = 0; q < NPT; ++q) {
    const int il = i0 + q;
    if (il < L) {
      const int k = r.list[sN + il];
      int code = 0;
#pragma unroll
      for (int j = 0; j < H; ++j) {
        if (j < nL) {
          const float v = Lf[q][j];
          if (bad_value(v, &code)) set_error(r, code, 1, s, k, e, j);
          Lf[q][j] = v < FLT_MIN ? FLT_MIN : v;
        }
        if (j < nR) {
          const float v = Rf[q][j];
          if (bad_value(v, &code)) set_error(r, code, 1, s, k, e, m0 + j);
          Rf[q][j] = v < FLT_MIN ? FLT_MIN : v;
        }
      }
      // node k and the thinned nodes that reference it (previous list node + 1 .. k)
      const int kfirst = (il == 0) ? 0 : r.list[sN + il - 1] + 1;
      for (int kk = kfirst; kk <= k; ++kk) {
        float *op = reinterpret_cast<float *>(r.f) + ((sN + kk) * r.E + e) * M;
#pragma unroll
        for (int j = 0; j < H; ++j) {
          if (j < nL) op[j] = Lf[q][j];
          if (j < nR) op[m0 + j] = Rf[q][j];
        }
        r.fexp[(sN + kk) * r.E + e] = (short)K;
      }
    }
  }
  if (C > 1) cluster.sync();
}

// The packed shapes: the upwind and relaxation arithmetic on pairs of mu
// cells with the packed fp32x2 instructions (two cells per instruction, the
// same roundings as the scalar fused multiply-adds of k_stream2).  f is held
// as pairs (float2) from load to store, so every pair sits in an aligned
// register pair.  FILLED: both halves
// fill their MMAX/2 slots (M = MMAX, m0 = M/2), every cell guard is known at
// compile time and rows move as float4 (MMAX is a multiple of 8: 16-byte
// aligned rows).  Otherwise rows move cell by cell under run-time guards,
// and a half with an odd number of cells is padded at slot 0 with a cell
// held at zero: its upwind value stays 0 (0 + c (0 - 0), the neighbours'
// padding is zero too), it adds nothing to the isotropisation sum, and it is
// zeroed again after the seed boundary and the relaxation set it.
// One (stream s, energy e) slab of run r, on a CTA (or cluster) of T
// threads: the body of k_stream2_pairs and of k_stream2_pairs_multi.
template <int MMAX, int T, int NPT, bool FILLED>
__device__ __forceinline__ void stream2_pairs_slab(const RunView &r, const int s, const int e,
                                                   int m0) {
  constexpr int W = T / 32;
  constexpr int H = MMAX / 2;  // cells per direction
  constexpr int P = H / 2;     // pairs per direction
  static_assert(H % 4 == 0, "rows move as float4");
  constexpr unsigned FULL = 0xffffffffu;
  extern __shared__ __align__(16) float halo[];  // [p][hi/lo][W+1][H]
  auto hi = [&](int p, int w) { return halo + ((p * 2 + 0) * (W + 1) + w) * H; };
  auto lo = [&](int p, int w) { return halo + ((p * 2 + 1) * (W + 1) + w) * H; };

  cg::cluster_group cluster = cg::this_cluster();
  const int C = (int)cluster.num_blocks();
  const int crank = (int)cluster.block_rank();
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int N = r.N;
  const int M = FILLED ? MMAX : r.M;
  if (FILLED) m0 = H;
  const int shL = FILLED ? 0 : (m0 & 1), shR = FILLED ? 0 : ((M - m0) & 1);  // padding
  const int nPL = FILLED ? P : (m0 + shL) / 2, nPR = FILLED ? P : (M - m0 + shR) / 2;
  const int L = r.list_size[s];
  if (L < 3) return;

  const EnergyConsts ec = r.ec[e];
  const double dtMin = 0.4 * r.ds_min[s] * ec.vgrid_i;
  const double nst = floor(r.dt / dtMin + 1.0);
  if (!(nst <= (double)r.max_subcycles)) {
    if (crank == 0 && tid == 0) set_error(r, EPREM_GPU_ERR_SUBCYCLES, 1, s, -1, e, -1);
    return;
  }
  const int nsteps = (int)nst;
  const double dtProp = r.dt / (1.0 * nsteps);
  if (crank == 0 && tid == 0) {
    atomicMax(&r.status->max_stream, nsteps);
    atomicAdd(&r.status->stream_cs, (unsigned long long)nsteps * L * M);
  }
  for (int j = tid; j < 2 * 2 * (W + 1) * H; j += T) halo[j] = 0.f;

  const int i0 = NPT * (crank * T + tid);
  const size_t sN = (size_t)s * N;
  float2 Lf[NPT][P], Rf[NPT][P];  // mu = 2p, 2p+1 and m0 + 2p, m0 + 2p + 1
  float2 mhi[NPT], mlo[NPT];
  float phi[NPT], omlo[NPT], dith[NPT];
  __shared__ float s_bcv[3];
  __shared__ int s_red[W + 1];
  const double vdt = ec.vgrid * dtProp;
  const float4 *cf = r.scoef + ((size_t)s * r.E + e) * N;
  int xr[NPT];      // the rows' exponents as loaded
  float sw[NPT];    // seed * 2^seed_k
  int lg = kNoExp;  // largest floor(log2) of a true value of this thread's rows and seeds
#pragma unroll
  for (int q = 0; q < NPT; ++q) {
    mhi[q] = mlo[q] = make_float2(0.f, 0.f);
    phi[q] = omlo[q] = 0.f;
    dith[q] = 0.5f;
    xr[q] = 0;
    sw[q] = 0.f;
#pragma unroll
    for (int p = 0; p < P; ++p) Lf[q][p] = Rf[q][p] = make_float2(0.f, 0.f);
    const int il = i0 + q;
    if (il < L) {
      const int k = r.list[sN + il];
      const float4 c = cf[il];
      const float *row = reinterpret_cast<const float *>(r.f) + ((sN + k) * r.E + e) * M;
      if constexpr (FILLED) {
        const float4 *fp = reinterpret_cast<const float4 *>(row);
#pragma unroll
        for (int t = 0; t < P / 2; ++t) {
          const float4 a = fp[t], b = fp[H / 4 + t];
          Lf[q][2 * t] = make_float2(a.x, a.y);
          Lf[q][2 * t + 1] = make_float2(a.z, a.w);
          Rf[q][2 * t] = make_float2(b.x, b.y);
          Rf[q][2 * t + 1] = make_float2(b.z, b.w);
        }
      } else {  // slot j holds cell j - sh of its half
#pragma unroll
        for (int t = 0; t < P; ++t) {
          if (t < nPL) {
            if (t > 0 || !shL) Lf[q][t].x = row[2 * t - shL];
            Lf[q][t].y = row[2 * t + 1 - shL];
          }
          if (t < nPR) {
            if (t > 0 || !shR) Rf[q][t].x = row[m0 + 2 * t - shR];
            Rf[q][t].y = row[m0 + 2 * t + 1 - shR];
          }
        }
      }
      float mx = 0.f;  // padding cells are zero
#pragma unroll
      for (int t = 0; t < P; ++t)
        mx = fmaxf(mx, fmaxf(fmaxf(Lf[q][t].x, Lf[q][t].y), fmaxf(Rf[q][t].x, Rf[q][t].y)));
      xr[q] = r.fexp[(sN + k) * r.E + e];
      sw[q] = c.w;
      const int lr = ilogb_f(mx);
      if (lr != kNoExp) lg = max(lg, lr - xr[q]);
      const int ls = ilogb_f(c.w);
      if ((r.check_seed || (r.use_bc && il < 3)) && ls != kNoExp) lg = max(lg, ls - ec.seed_k);
      const float mh = (il == 0) ? 0.f : c.x, ml = (il == L - 1) ? 0.f : c.x;
      mhi[q] = make_float2(mh, mh);
      mlo[q] = make_float2(ml, ml);
      phi[q] = c.y;
      omlo[q] = c.z;
    }
  }
  // the slab's common exponent; rows and seeds brought to it (exact powers of two)
  const int K = slab_exp<T>(lg, s_red, cluster, C);
#pragma unroll
  for (int q = 0; q < NPT; ++q) {
    const int il = i0 + q;
    if (il < L) {
      const Pow2Pair pf = pow2_pair(K - xr[q]);
      const float seedf = scale2(sw[q], pow2_pair(K - ec.seed_k));
#pragma unroll
      for (int t = 0; t < P; ++t) {
        Lf[q][t] = make_float2(scale2(Lf[q][t].x, pf), scale2(Lf[q][t].y, pf));
        Rf[q][t] = make_float2(scale2(Rf[q][t].x, pf), scale2(Rf[q][t].y, pf));
      }
      if (r.check_seed) {  // seedPopulationCheck (scaled alike: the same order); padding stays 0
#pragma unroll
        for (int t = 0; t < P; ++t) {
          if (FILLED || t < nPL) {
            if (t > 0 || !shL) Lf[q][t].x = Lf[q][t].x < seedf ? seedf : Lf[q][t].x;
            Lf[q][t].y = Lf[q][t].y < seedf ? seedf : Lf[q][t].y;
          }
          if (FILLED || t < nPR) {
            if (t > 0 || !shR) Rf[q][t].x = Rf[q][t].x < seedf ? seedf : Rf[q][t].x;
            Rf[q][t].y = Rf[q][t].y < seedf ? seedf : Rf[q][t].y;
          }
        }
      }
      if (il < 3) s_bcv[il] = seedf;
    }
  }
  // del of slot j: vdt mugrid(cell j - sh) = (first cell's del - sh ddel) + j ddel
  const float ddel = (float)(vdt * r.dmu);
  const float dl0 = (float)(vdt * r.mugrid[0]) - (float)shL * ddel;
  const float dr0 = (float)(vdt * r.mugrid[m0 < M ? m0 : M - 1]) - (float)shR * ddel;
  const float inv_m = (float)(1.0 / M);
  float *next_hi0 = (C > 1 && crank < C - 1) ? cluster.map_shared_rank(halo, crank + 1) : nullptr;
  float *prev_loW = (C > 1 && crank > 0) ? cluster.map_shared_rank(halo, crank - 1) : nullptr;
  if (C > 1)
    cluster.sync();
  else
    __syncthreads();

  const float2 neg1 = make_float2(-1.f, -1.f);
  for (int step = 0; step < nsteps; ++step) {
    const int ph = step & 1;
    if (r.use_bc && crank == 0 && warp == 0) {  // list nodes 0..2 live in warp 0
#pragma unroll
      for (int q = 0; q < NPT; ++q) {
        if (i0 + q < 3) {
          const float b = s_bcv[i0 + q];
#pragma unroll
          for (int p = 0; p < P; ++p) Lf[q][p] = Rf[q][p] = make_float2(b, b);
          if (shL) Lf[q][0].x = 0.f;  // padding
          if (shR) Rf[q][0].x = 0.f;
        }
      }
    }
    if (lane == 31) {  // last node's outward half for the next warp's first node
      float4 *dst = reinterpret_cast<float4 *>(hi(ph, warp + 1));
      float4 *rdst = (warp == W - 1 && next_hi0)
                         ? reinterpret_cast<float4 *>(next_hi0 + ((ph * 2 + 0) * (W + 1)) * H)
                         : nullptr;
      if constexpr (FILLED) {
#pragma unroll
        for (int t = 0; t < P / 2; ++t) {
          const float4 v = make_float4(Rf[NPT - 1][2 * t].x, Rf[NPT - 1][2 * t].y,
                                       Rf[NPT - 1][2 * t + 1].x, Rf[NPT - 1][2 * t + 1].y);
          dst[t] = v;
          if (rdst) rdst[t] = v;
        }
      } else {
        float2 *d2 = reinterpret_cast<float2 *>(dst), *r2 = reinterpret_cast<float2 *>(rdst);
#pragma unroll
        for (int t = 0; t < P; ++t)
          if (t < nPR) {
            d2[t] = Rf[NPT - 1][t];
            if (r2) r2[t] = Rf[NPT - 1][t];
          }
      }
    }
    if (lane == 0) {  // first node's inward half for the previous warp's last node
      float4 *dst = reinterpret_cast<float4 *>(lo(ph, warp));
      float4 *rdst = (warp == 0 && prev_loW)
                         ? reinterpret_cast<float4 *>(prev_loW + ((ph * 2 + 1) * (W + 1) + W) * H)
                         : nullptr;
      if constexpr (FILLED) {
#pragma unroll
        for (int t = 0; t < P / 2; ++t) {
          const float4 v = make_float4(Lf[0][2 * t].x, Lf[0][2 * t].y, Lf[0][2 * t + 1].x,
                                       Lf[0][2 * t + 1].y);
          dst[t] = v;
          if (rdst) rdst[t] = v;
        }
      } else {
        float2 *d2 = reinterpret_cast<float2 *>(dst), *r2 = reinterpret_cast<float2 *>(rdst);
#pragma unroll
        for (int t = 0; t < P; ++t)
          if (t < nPL) {
            d2[t] = Lf[0][t];
            if (r2) r2[t] = Lf[0][t];
          }
      }
    }
    if (C > 1)
      cluster.sync();
    else
      __syncthreads();
    const float2 *my_hi = reinterpret_cast<const float2 *>(hi(ph, warp));
    const float2 *my_lo = reinterpret_cast<const float2 *>(lo(ph, warp + 1));
    float2 acc[NPT];
#pragma unroll
    for (int q = 0; q < NPT; ++q) acc[q] = make_float2(0.f, 0.f);
    // mu < 0: upwind from the outer neighbour (list node + 1), old values
#pragma unroll
    for (int p = 0; p < P; ++p) {
      if (!FILLED && p >= nPL) continue;
      float d0 = dl0 + (float)(2 * p) * ddel, d1 = dl0 + (float)(2 * p + 1) * ddel;
      // opaque to loop-invariant code motion: otherwise every mult*del product
      // is hoisted out of the sub-cycle loop into registers
      asm volatile("" : "+f"(d0), "+f"(d1));
      const float2 del2 = make_float2(d0, d1);
      float2 nb;
      nb.x = __shfl_down_sync(FULL, Lf[0][p].x, 1);
      nb.y = __shfl_down_sync(FULL, Lf[0][p].y, 1);
      if (lane == 31) nb = my_lo[p];
#pragma unroll
      for (int q = 0; q < NPT; ++q) {
        const float2 cur = Lf[q][p];
        const float2 right = (q + 1 < NPT) ? Lf[q + 1 < NPT ? q + 1 : q][p] : nb;
        const float2 nw = __ffma2_rn(__fmul2_rn(mlo[q], del2), __ffma2_rn(right, neg1, cur), cur);
        Lf[q][p] = nw;
        acc[q] = __fadd2_rn(acc[q], nw);
      }
    }
    // mu >= 0: upwind from the inner neighbour (list node - 1), old values
#pragma unroll
    for (int p = 0; p < P; ++p) {
      if (!FILLED && p >= nPR) continue;
      float d0 = dr0 + (float)(2 * p) * ddel, d1 = dr0 + (float)(2 * p + 1) * ddel;
      asm volatile("" : "+f"(d0), "+f"(d1));
      const float2 del2 = make_float2(d0, d1);
      float2 nb;
      nb.x = __shfl_up_sync(FULL, Rf[NPT - 1][p].x, 1);
      nb.y = __shfl_up_sync(FULL, Rf[NPT - 1][p].y, 1);
      if (lane == 0) nb = my_hi[p];
#pragma unroll
      for (int q = NPT - 1; q >= 0; --q) {
        const float2 cur = Rf[q][p];
        const float2 left = (q > 0) ? Rf[q > 0 ? q - 1 : 0][p] : nb;
        const float2 nw = __ffma2_rn(__fmul2_rn(mhi[q], del2), __ffma2_rn(cur, neg1, left), cur);
        Rf[q][p] = nw;
        acc[q] = __fadd2_rn(acc[q], nw);
      }
    }
#pragma unroll
    for (int q = 0; q < NPT; ++q) {
      const float om = relax_weight(omlo[q], phi[q], dith[q]), em = 1.f - om;
      const float iso = (inv_m * (acc[q].x + acc[q].y)) * om;
      const float2 iso2 = make_float2(iso, iso), em2 = make_float2(em, em);
#pragma unroll
      for (int p = 0; p < P; ++p) {
        Lf[q][p] = __ffma2_rn(Lf[q][p], em2, iso2);
        Rf[q][p] = __ffma2_rn(Rf[q][p], em2, iso2);
      }
    }
    if (!FILLED && (shL | shR)) {  // padding back to zero (uniform branch)
#pragma unroll
      for (int q = 0; q < NPT; ++q) {
        if (shL) Lf[q][0].x = 0.f;
        if (shR) Rf[q][0].x = 0.f;
      }
    }
  }

#pragma unroll
  for (int q = 0; q < NPT; ++q) {
    const int il = i0 + q;
    if (il < L) {
      const int k = r.list[sN + il];
      int code = 0;
#pragma unroll
      for (int p = 0; p < P; ++p) {
        float2 a = Lf[q][p], b = Rf[q][p];
        if (FILLED || p < nPL) {
          if ((p > 0 || !shL) && bad_value(a.x, &code))
            set_error(r, code, 1, s, k, e, 2 * p - shL);
          if (bad_value(a.y, &code)) set_error(r, code, 1, s, k, e, 2 * p + 1 - shL);
        }
        if (FILLED || p < nPR) {
          if ((p > 0 || !shR) && bad_value(b.x, &code))
            set_error(r, code, 1, s, k, e, m0 + 2 * p - shR);
          if (bad_value(b.y, &code)) set_error(r, code, 1, s, k, e, m0 + 2 * p + 1 - shR);
        }
        a.x = a.x < FLT_MIN ? FLT_MIN : a.x; a.y = a.y < FLT_MIN ? FLT_MIN : a.y;
        b.x = b.x < FLT_MIN ? FLT_MIN : b.x; b.y = b.y < FLT_MIN ? FLT_MIN : b.y;
        Lf[q][p] = a;
        Rf[q][p] = b;
      }
      // node k and the thinned nodes that reference it (previous list node + 1 .. k)
      const int kfirst = (il == 0) ? 0 : r.list[sN + il - 1] + 1;
      for (int kk = kfirst; kk <= k; ++kk) {
        r.fexp[(sN + kk) * r.E + e] = (short)K;
        float *row = reinterpret_cast<float *>(r.f) + ((sN + kk) * r.E + e) * M;
        if constexpr (FILLED) {
          float4 *op = reinterpret_cast<float4 *>(row);
#pragma unroll
          for (int t = 0; t < P / 2; ++t) {
            op[t] = make_float4(Lf[q][2 * t].x, Lf[q][2 * t].y, Lf[q][2 * t + 1].x,
                                Lf[q][2 * t + 1].y);
            op[H / 4 + t] = make_float4(Rf[q][2 * t].x, Rf[q][2 * t].y, Rf[q][2 * t + 1].x,
                                        Rf[q][2 * t + 1].y);
          }
        } else {
#pragma unroll
          for (int t = 0; t < P; ++t) {
            if (t < nPL) {
              if (t > 0 || !shL) row[2 * t - shL] = Lf[q][t].x;
              row[2 * t + 1 - shL] = Lf[q][t].y;
            }
            if (t < nPR) {
              if (t > 0 || !shR) row[m0 + 2 * t - shR] = Rf[q][t].x;
              row[m0 + 2 * t + 1 - shR] = Rf[q][t].y;
            }
          }
        }
      }
    }
  }
  if (C > 1) cluster.sync();
}

template <int MMAX, int T, int NPT, bool FILLED>
__global__ void __launch_bounds__(T, 1) k_stream2_pairs(RunView r, int m0) {
  stream2_pairs_slab<MMAX, T, NPT, FILLED>(r, blockIdx.y, r.E - 1 - (int)blockIdx.z, m0);
}

// The same kernel over the slabs of several runs in one launch (batched
// ensembles): cluster i of the launch takes slab items[i] = (run, stream,
// energy), the items in decreasing order of estimated work, so the slabs of
// small runs fill the tail of the large ones.  Every slab is computed as the
// one-run launch computes it.
template <int MMAX, int T, int NPT, bool FILLED>
__global__ void __launch_bounds__(T, 1)
    k_stream2_pairs_multi(const __grid_constant__ MultiRunViews mv, const int4 *items) {
  cg::cluster_group cluster = cg::this_cluster();
  const int4 it = items[blockIdx.x / cluster.num_blocks()];
  // the run's view stays in the parameter bank (indexed constant loads)
  stream2_pairs_slab<MMAX, T, NPT, FILLED>(mv.v[it.x], it.y, it.z, mv.m0[it.x]);
}

// The mirrored shapes (kinds 6 and 7): the packed shape with every cell guard
// known at compile time (M = MMAX, m0 = M/2), with the mu < 0 half held in
// mirror order -- slot j of that half is cell H-1-j, whose |mugrid| is that of
// cell H+j on the uniform mu grid -- so that pair p of either half moves with
// the same upwind coefficient c = mult |v dtProp mugrid|, written for the
// mu < 0 half as f + c (f[+1] - f) (the reference's f + mult del (f - f[+1])
// with del < 0, src/energeticParticles.c:2392-2397).  Per cell and sub-cycle
// that leaves the difference, the update, the sum and the relaxation on the
// FMA pipe.  Kind 7 forms the coefficients once per launch into shared memory
// (float4 [P/2][NPT][T], or float2 [P][NPT][T] when M/2 is not a multiple of
// 4; on the sub-cycle loop one 8-byte load per node and pair index serves a
// pair of cells of each half); kind 6 forms them on the loop (one packed
// multiply per node and pair index, shared by the two halves).
// The two ends of the stream keep their values without a zero multiplier:
//   * list node 0, mu >= 0 (:2380): with the seed boundary, node 0 holds the
//     seed at the upwind step, and so does its upwind neighbour -- the empty
//     slots in front of it, which the boundary sets alike, or the first halo
//     row, set to the seed once per launch -- so its difference is zero;
//   * the last list node, mu < 0 (:2391): the slots are shifted so that it is
//     the last node of its thread, which publishes its mu < 0 half each
//     sub-cycle with the halo rows and reads it back as its neighbour.
// So these kinds need the seed boundary and N + NPT - 1 slots.
template <int MMAX, int T, int NPT, bool CSM>
constexpr size_t stream2_mirror_smem_bytes() {
  return stream2_smem_bytes<MMAX, T>() + sizeof(float) * 2 * (MMAX / 2) +
         (CSM ? sizeof(float2) * (MMAX / 4) * NPT * T : 0);
}

// A half row of P pairs to shared memory (and to a second, possibly remote,
// copy): as float4 when V4, else as float2.
template <int P, bool V4>
__device__ __forceinline__ void put_half(const float2 (&h)[P], float *dst, float *dst2) {
  if constexpr (V4) {
#pragma unroll
    for (int t = 0; t < P / 2; ++t) {
      const float4 v = make_float4(h[2 * t].x, h[2 * t].y, h[2 * t + 1].x, h[2 * t + 1].y);
      reinterpret_cast<float4 *>(dst)[t] = v;
      if (dst2) reinterpret_cast<float4 *>(dst2)[t] = v;
    }
  } else {
#pragma unroll
    for (int t = 0; t < P; ++t) {
      reinterpret_cast<float2 *>(dst)[t] = h[t];
      if (dst2) reinterpret_cast<float2 *>(dst2)[t] = h[t];
    }
  }
}

// Bounded wait on a CTA mbarrier phase: at most kMirrorWaitLimit try_waits,
// each of which suspends the warp until the phase completes or about a
// microsecond has passed; false when the limit ran out.  (Publishing the
// warp-edge rows right after relaxing the edge nodes, before the others, and
// a few test_wait polls before suspending measured slower: 8.00 against
// 7.75 ms per 96-stream launch, the reordering spilling registers.)
constexpr int kMirrorWaitLimit = 1 << 20;
__device__ __forceinline__ bool halo_wait(uint64_t *bar, uint32_t parity) {
  const uint32_t a = (uint32_t)__cvta_generic_to_shared(bar);
  for (int i = 0; i < kMirrorWaitLimit; i++) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity), "r"(1000u)
        : "memory");
    if (done) return true;
  }
  return false;
}
// put_half and halo_arrive by the lanes where p holds, as predicated
// instructions of the whole warp rather than a divergent branch.
template <int P, bool V4>
__device__ __forceinline__ void put_half_if(bool p, const float2 (&h)[P], float *dst) {
  const uint32_t a = (uint32_t)__cvta_generic_to_shared(dst);
  const uint32_t pr = p ? 1u : 0u;
  if constexpr (V4) {
#pragma unroll
    for (int t = 0; t < P / 2; ++t)
      asm volatile(
          "{\n .reg .pred q;\n setp.ne.u32 q, %0, 0;\n"
          " @q st.shared.v4.f32 [%1], {%2, %3, %4, %5};\n}\n" ::"r"(pr),
          "r"(a + 16u * t), "f"(h[2 * t].x), "f"(h[2 * t].y), "f"(h[2 * t + 1].x),
          "f"(h[2 * t + 1].y)
          : "memory");
  } else {
#pragma unroll
    for (int t = 0; t < P; ++t)
      asm volatile(
          "{\n .reg .pred q;\n setp.ne.u32 q, %0, 0;\n"
          " @q st.shared.v2.f32 [%1], {%2, %3};\n}\n" ::"r"(pr),
          "r"(a + 8u * t), "f"(h[t].x), "f"(h[t].y)
          : "memory");
  }
}
__device__ __forceinline__ void halo_arrive_if(bool p, uint64_t *bar) {
  const uint32_t a = (uint32_t)__cvta_generic_to_shared(bar);
  asm volatile(
      "{\n .reg .pred q;\n .reg .b64 st;\n setp.ne.u32 q, %0, 0;\n"
      " @q mbarrier.arrive.shared::cta.b64 st, [%1];\n}\n" ::"r"(p ? 1u : 0u),
      "r"(a)
      : "memory");
}
__device__ __forceinline__ void halo_arrive(uint64_t *bar) {
  const uint32_t a = (uint32_t)__cvta_generic_to_shared(bar);
  asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.shared::cta.b64 st, [%0];\n}\n" ::"r"(a)
               : "memory");
}
// ASYNC (1, one CTA per slab; 0: a CTA or cluster barrier per sub-cycle):
// instead of a CTA barrier per sub-cycle, each warp waits only for the halo
// rows of its two neighbour warps -- an mbarrier per (parity, warp) that lane
// 31 of the warp before and lane 0 of the warp after arrive on once their
// rows are stored (release / acquire at CTA scope).  Warps then drift up to
// one sub-cycle apart; the two parities of the halo rows cover that: a warp
// writes a parity's row again only after its neighbour has published the
// next sub-cycle, i.e. has read the row.  Across the CTAs of a cluster the
// same hand-over (remote arrivals at cluster scope) measured no faster than
// the cluster barrier: 15.02 against 14.88 ms per 96-stream launch at
// N = 1500, whose 128-thread CTAs share an SM two by two, so one CTA's
// barrier wait overlaps the other's work.
template <int MMAX, int T, int NPT, bool CSM, int ASYNC>
__device__ __forceinline__ void stream2_mirror_slab(const RunView &r, const int s, const int e) {
  constexpr int W = T / 32;
  constexpr int H = MMAX / 2;  // cells per direction
  constexpr int P = H / 2;     // pairs per direction
  constexpr int M = MMAX;
  static_assert(H % 2 == 0, "rows move as float2 pairs");
  constexpr bool V4 = H % 4 == 0;  // rows, halo rows and coefficients as float4
  constexpr unsigned FULL = 0xffffffffu;
  // [p][hi/lo][W+1][H] halo rows, then [p][H] the last node's own row, then
  // (kind 7) the coefficients [P/2][NPT][T]
  extern __shared__ __align__(16) float halo[];
  auto hi = [&](int p, int w) { return halo + ((p * 2 + 0) * (W + 1) + w) * H; };
  auto lo = [&](int p, int w) { return halo + ((p * 2 + 1) * (W + 1) + w) * H; };
  float *self = halo + 2 * 2 * (W + 1) * H;
  float *csm = self + 2 * H;  // V4: float4 [P/2][NPT][T], else float2 [P][NPT][T]

  cg::cluster_group cluster = cg::this_cluster();
  const int C = (int)cluster.num_blocks();
  const int crank = (int)cluster.block_rank();
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int N = r.N;
  const int L = r.list_size[s];
  if (L < 3) return;

  const EnergyConsts ec = r.ec[e];
  const double dtMin = 0.4 * r.ds_min[s] * ec.vgrid_i;
  const double nst = floor(r.dt / dtMin + 1.0);
  if (!(nst <= (double)r.max_subcycles)) {
    if (crank == 0 && tid == 0) set_error(r, EPREM_GPU_ERR_SUBCYCLES, 1, s, -1, e, -1);
    return;
  }
  const int nsteps = (int)nst;
  const double dtProp = r.dt / (1.0 * nsteps);
  if (crank == 0 && tid == 0) {
    atomicMax(&r.status->max_stream, nsteps);
    atomicAdd(&r.status->stream_cs, (unsigned long long)nsteps * L * M);
  }
  for (int j = tid; j < 2 * 2 * (W + 1) * H + 2 * H; j += T) halo[j] = 0.f;
  __shared__ uint64_t s_bar[2][W];  // ASYNC: [parity][warp], arrivals of the neighbour warps
  if (ASYNC && tid < 2 * W) {  // writers: the warps before and after
    const int w = tid % W, cnt = (w > 0) + (w < W - 1);
    if (cnt)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(
                       (uint32_t)__cvta_generic_to_shared(&s_bar[tid / W][w])),
                   "r"(cnt)
                   : "memory");
  }  // made visible by the barriers before the sub-cycle loop

  // list node of this thread's first slot: the slots start sh < NPT nodes
  // before list node 0, so that node L-1 is the last node of its thread
  const int sh = (NPT - L % NPT) % NPT;
  const int i0 = NPT * (crank * T + tid) - sh;
  const bool is_last = i0 + NPT - 1 == L - 1;
  const size_t sN = (size_t)s * N;
  // Lf pair p: cells H-1-2p, H-2-2p (mirror order); Rf pair p: cells H+2p, H+2p+1
  float2 Lf[NPT][P], Rf[NPT][P];
  float2 m2[NPT];
  float phi[NPT], omlo[NPT], dith[NPT];
  __shared__ float s_bcv[3];
  __shared__ int s_red[W + 1];
  const double vdt = ec.vgrid * dtProp;
  const float4 *cf = r.scoef + ((size_t)s * r.E + e) * N;
  int xr[NPT];
  float sw[NPT];
  int lg = kNoExp;
#pragma unroll
  for (int q = 0; q < NPT; ++q) {
    m2[q] = make_float2(0.f, 0.f);
    phi[q] = omlo[q] = 0.f;
    dith[q] = 0.5f;
    xr[q] = 0;
    sw[q] = 0.f;
#pragma unroll
    for (int p = 0; p < P; ++p) Lf[q][p] = Rf[q][p] = make_float2(0.f, 0.f);
    const int il = i0 + q;
    if (il >= 0 && il < L) {
      const int k = r.list[sN + il];
      const float4 c = cf[il];
      const float *row = reinterpret_cast<const float *>(r.f) + ((sN + k) * r.E + e) * M;
      if constexpr (V4) {
        const float4 *fp = reinterpret_cast<const float4 *>(row);
#pragma unroll
        for (int t = 0; t < P / 2; ++t) {
          const float4 a = fp[t], b = fp[H / 4 + t];
          Lf[q][P - 1 - 2 * t] = make_float2(a.y, a.x);
          Lf[q][P - 2 - 2 * t] = make_float2(a.w, a.z);
          Rf[q][2 * t] = make_float2(b.x, b.y);
          Rf[q][2 * t + 1] = make_float2(b.z, b.w);
        }
      } else {
        const float2 *fp = reinterpret_cast<const float2 *>(row);
#pragma unroll
        for (int t = 0; t < P; ++t) {
          const float2 a = fp[t];
          Lf[q][P - 1 - t] = make_float2(a.y, a.x);
          Rf[q][t] = fp[H / 2 + t];
        }
      }
      float mx = 0.f;
#pragma unroll
      for (int t = 0; t < P; ++t)
        mx = fmaxf(mx, fmaxf(fmaxf(Lf[q][t].x, Lf[q][t].y), fmaxf(Rf[q][t].x, Rf[q][t].y)));
      xr[q] = r.fexp[(sN + k) * r.E + e];
      sw[q] = c.w;
      const int lr = ilogb_f(mx);
      if (lr != kNoExp) lg = max(lg, lr - xr[q]);
      const int ls = ilogb_f(c.w);
      if ((r.check_seed || il < 3) && ls != kNoExp) lg = max(lg, ls - ec.seed_k);
      m2[q] = make_float2(c.x, c.x);
      phi[q] = c.y;
      omlo[q] = c.z;
    }
  }
  const int K = slab_exp<T>(lg, s_red, cluster, C);
#pragma unroll
  for (int q = 0; q < NPT; ++q) {
    const int il = i0 + q;
    if (il >= 0 && il < L) {
      const Pow2Pair pf = pow2_pair(K - xr[q]);
      const float seedf = scale2(sw[q], pow2_pair(K - ec.seed_k));
#pragma unroll
      for (int t = 0; t < P; ++t) {
        Lf[q][t] = make_float2(scale2(Lf[q][t].x, pf), scale2(Lf[q][t].y, pf));
        Rf[q][t] = make_float2(scale2(Rf[q][t].x, pf), scale2(Rf[q][t].y, pf));
      }
      if (r.check_seed) {
#pragma unroll
        for (int t = 0; t < P; ++t) {
          Lf[q][t].x = Lf[q][t].x < seedf ? seedf : Lf[q][t].x;
          Lf[q][t].y = Lf[q][t].y < seedf ? seedf : Lf[q][t].y;
          Rf[q][t].x = Rf[q][t].x < seedf ? seedf : Rf[q][t].x;
          Rf[q][t].y = Rf[q][t].y < seedf ? seedf : Rf[q][t].y;
        }
      }
      if (il < 3) s_bcv[il] = seedf;
    }
  }
  // |del| of pair p of either half: v dtProp mugrid of cells H+2p, H+2p+1
  const float ddel = (float)(vdt * r.dmu);
  const float d0 = (float)(vdt * r.mugrid[H]);
  if constexpr (CSM) {  // this thread's own coefficients: no barrier needed
#pragma unroll
    for (int p = 0; p < P; ++p) {
#pragma unroll
      for (int q = 0; q < NPT; ++q) {
        const float m = m2[q].x;
        const float2 c = make_float2(m * (d0 + (float)(2 * p) * ddel),
                                     m * (d0 + (float)(2 * p + 1) * ddel));
        if constexpr (V4)
          reinterpret_cast<float2 *>(reinterpret_cast<float4 *>(csm) +
                                     ((p >> 1) * NPT + q) * T + tid)[p & 1] = c;
        else
          reinterpret_cast<float2 *>(csm)[(p * NPT + q) * T + tid] = c;
      }
    }
  }
  const float inv_m = (float)(1.0 / M);
  float *next_hi0 = (C > 1 && crank < C - 1) ? cluster.map_shared_rank(halo, crank + 1) : nullptr;
  float *prev_loW = (C > 1 && crank > 0) ? cluster.map_shared_rank(halo, crank - 1) : nullptr;
  if (C > 1)
    cluster.sync();
  else
    __syncthreads();
  if (crank == 0 && tid == 0) {  // list node 0's upwind neighbour for mu >= 0: the seed
    const float b = s_bcv[0];
    for (int j = 0; j < H; ++j) hi(0, 0)[j] = hi(1, 0)[j] = b;
  }

  const float2 neg1 = make_float2(-1.f, -1.f);
  bool timed_out = false;
  // the warp-edge rows of sub-cycle parity p: lane 31's outward half for the
  // next warp's first node, lane 0's inward half (mirror order) for the
  // previous warp's last node; with ASYNC, each followed by the arrival its
  // reader waits on (the seed boundary is set before: list nodes 0..2 sit in
  // threads 0 and 1)
  auto publish_edges = [&](int p) {
    if constexpr (ASYNC == 1) {  // one CTA: predicated stores and arrivals, no branch
      put_half_if<P, V4>(lane == 31, Rf[NPT - 1], hi(p, warp + 1));
      halo_arrive_if(lane == 31 && warp + 1 < W, &s_bar[p][warp + 1 < W ? warp + 1 : 0]);
      put_half_if<P, V4>(lane == 0, Lf[0], lo(p, warp));
      halo_arrive_if(lane == 0 && warp > 0, &s_bar[p][warp > 0 ? warp - 1 : 0]);
      return;
    }
    if (lane == 31) {
      put_half<P, V4>(Rf[NPT - 1], hi(p, warp + 1),
                      (warp == W - 1 && next_hi0) ? next_hi0 + ((p * 2 + 0) * (W + 1)) * H
                                                  : nullptr);
      if (ASYNC && warp + 1 < W) halo_arrive(&s_bar[p][warp + 1]);
    }
    if (lane == 0) {
      put_half<P, V4>(Lf[0], lo(p, warp),
                      (warp == 0 && prev_loW) ? prev_loW + ((p * 2 + 1) * (W + 1) + W) * H
                                              : nullptr);
      if (ASYNC && warp > 0) halo_arrive(&s_bar[p][warp - 1]);
    }
  };
  for (int step = 0; step < nsteps; ++step) {
    const int ph = step & 1;
    if (crank == 0 && warp == 0) {  // seed boundary: list nodes 0..2 and the slots in front
#pragma unroll
      for (int q = 0; q < NPT; ++q) {
        const int il = i0 + q;
        if (il < 3) {
          const float b = s_bcv[il < 0 ? 0 : il];
#pragma unroll
          for (int p = 0; p < P; ++p) Lf[q][p] = Rf[q][p] = make_float2(b, b);
        }
      }
    }
    publish_edges(ph);
    if (is_last)  // the last list node is its own outer neighbour
      put_half<P, V4>(Lf[NPT - 1], self + ph * H, nullptr);
    if constexpr (ASYNC) {
      if (W > 1 && !timed_out && !halo_wait(&s_bar[ph][warp], (uint32_t)(step >> 1) & 1u)) {
        timed_out = true;  // reported once; later waits are skipped
        if (lane == 0) set_error(r, EPREM_GPU_ERR_CUDA, 1, s, -1, e, -1);
      }
    } else if (C > 1) {
      cluster.sync();
    } else {
      __syncthreads();
    }
    const float2 *my_hi = reinterpret_cast<const float2 *>(hi(ph, warp));
    const float2 *lo_src =
        reinterpret_cast<const float2 *>(is_last ? self + ph * H : lo(ph, warp + 1));
    const bool take_lo = is_last || lane == 31;
    float2 acc[NPT];
#pragma unroll
    for (int q = 0; q < NPT; ++q) acc[q] = make_float2(0.f, 0.f);
#pragma unroll
    for (int p = 0; p < P; ++p) {
      float2 c[NPT];
      if constexpr (CSM) {
#pragma unroll
        for (int q = 0; q < NPT; ++q) {
          if constexpr (V4)
            c[q] = reinterpret_cast<const float2 *>(reinterpret_cast<const float4 *>(csm) +
                                                    ((p >> 1) * NPT + q) * T + tid)[p & 1];
          else
            c[q] = reinterpret_cast<const float2 *>(csm)[(p * NPT + q) * T + tid];
        }
      } else {
        float dd0 = d0 + (float)(2 * p) * ddel, dd1 = d0 + (float)(2 * p + 1) * ddel;
        // opaque to loop-invariant code motion (see stream2_pairs_slab)
        asm volatile("" : "+f"(dd0), "+f"(dd1));
        const float2 del2 = make_float2(dd0, dd1);
#pragma unroll
        for (int q = 0; q < NPT; ++q) c[q] = __fmul2_rn(m2[q], del2);
      }
      float2 nbL, nbR;
      nbL.x = __shfl_down_sync(FULL, Lf[0][p].x, 1);
      nbL.y = __shfl_down_sync(FULL, Lf[0][p].y, 1);
      if (take_lo) nbL = lo_src[p];
      nbR.x = __shfl_up_sync(FULL, Rf[NPT - 1][p].x, 1);
      nbR.y = __shfl_up_sync(FULL, Rf[NPT - 1][p].y, 1);
      if (lane == 0) nbR = my_hi[p];
      // mu < 0: upwind from the outer neighbour (list node + 1), old values
#pragma unroll
      for (int q = 0; q < NPT; ++q) {
        const float2 cur = Lf[q][p];
        const float2 right = (q + 1 < NPT) ? Lf[q + 1 < NPT ? q + 1 : q][p] : nbL;
        const float2 nw = __ffma2_rn(c[q], __ffma2_rn(cur, neg1, right), cur);
        Lf[q][p] = nw;
        acc[q] = __fadd2_rn(acc[q], nw);
      }
      // mu >= 0: upwind from the inner neighbour (list node - 1), old values
#pragma unroll
      for (int q = NPT - 1; q >= 0; --q) {
        const float2 cur = Rf[q][p];
        const float2 left = (q > 0) ? Rf[q > 0 ? q - 1 : 0][p] : nbR;
        const float2 nw = __ffma2_rn(c[q], __ffma2_rn(cur, neg1, left), cur);
        Rf[q][p] = nw;
        acc[q] = __fadd2_rn(acc[q], nw);
      }
    }
#pragma unroll
    for (int q = 0; q < NPT; ++q) {
      const float om = relax_weight(omlo[q], phi[q], dith[q]), em = 1.f - om;
      const float iso = (inv_m * (acc[q].x + acc[q].y)) * om;
      const float2 iso2 = make_float2(iso, iso), em2 = make_float2(em, em);
#pragma unroll
      for (int p = 0; p < P; ++p) {
        Lf[q][p] = __ffma2_rn(Lf[q][p], em2, iso2);
        Rf[q][p] = __ffma2_rn(Rf[q][p], em2, iso2);
      }
    }
  }

#pragma unroll
  for (int q = 0; q < NPT; ++q) {
    const int il = i0 + q;
    if (il >= 0 && il < L) {
      const int k = r.list[sN + il];
      int code = 0;
#pragma unroll
      for (int p = 0; p < P; ++p) {
        float2 a = Lf[q][p], b = Rf[q][p];
        if (bad_value(a.x, &code)) set_error(r, code, 1, s, k, e, H - 1 - 2 * p);
        if (bad_value(a.y, &code)) set_error(r, code, 1, s, k, e, H - 2 - 2 * p);
        if (bad_value(b.x, &code)) set_error(r, code, 1, s, k, e, H + 2 * p);
        if (bad_value(b.y, &code)) set_error(r, code, 1, s, k, e, H + 2 * p + 1);
        a.x = a.x < FLT_MIN ? FLT_MIN : a.x; a.y = a.y < FLT_MIN ? FLT_MIN : a.y;
        b.x = b.x < FLT_MIN ? FLT_MIN : b.x; b.y = b.y < FLT_MIN ? FLT_MIN : b.y;
        Lf[q][p] = a;
        Rf[q][p] = b;
      }
      // node k and the thinned nodes that reference it (previous list node + 1 .. k)
      const int kfirst = (il == 0) ? 0 : r.list[sN + il - 1] + 1;
      for (int kk = kfirst; kk <= k; ++kk) {
        r.fexp[(sN + kk) * r.E + e] = (short)K;
        float *row = reinterpret_cast<float *>(r.f) + ((sN + kk) * r.E + e) * M;
        if constexpr (V4) {
          float4 *op = reinterpret_cast<float4 *>(row);
#pragma unroll
          for (int t = 0; t < P / 2; ++t) {
            op[t] = make_float4(Lf[q][P - 1 - 2 * t].y, Lf[q][P - 1 - 2 * t].x,
                                Lf[q][P - 2 - 2 * t].y, Lf[q][P - 2 - 2 * t].x);
            op[H / 4 + t] = make_float4(Rf[q][2 * t].x, Rf[q][2 * t].y, Rf[q][2 * t + 1].x,
                                        Rf[q][2 * t + 1].y);
          }
        } else {
          float2 *op = reinterpret_cast<float2 *>(row);
#pragma unroll
          for (int t = 0; t < P; ++t) {
            op[t] = make_float2(Lf[q][P - 1 - t].y, Lf[q][P - 1 - t].x);
            op[H / 2 + t] = Rf[q][t];
          }
        }
      }
    }
  }
  if (C > 1) cluster.sync();
}

template <int MMAX, int T, int NPT, bool CSM, int ASYNC>
__global__ void __launch_bounds__(T, 1) k_stream2_mirror(RunView r, int) {
  stream2_mirror_slab<MMAX, T, NPT, CSM, ASYNC>(r, blockIdx.y, r.E - 1 - (int)blockIdx.z);
}

template <int MMAX, int T, int NPT, bool CSM, int ASYNC>
__global__ void __launch_bounds__(T, 1)
    k_stream2_mirror_multi(const __grid_constant__ MultiRunViews mv, const int4 *items) {
  cg::cluster_group cluster = cg::this_cluster();
  const int4 it = items[blockIdx.x / cluster.num_blocks()];
  stream2_mirror_slab<MMAX, T, NPT, CSM, ASYNC>(mv.v[it.x], it.y, it.z);
}

// Per (stream, energy, list node): mult = ds_i min(tau / dtProp, 1), the
// relaxation factor exp(-dtProp / tau) and 1 - it, and the seed times
// 2^seed_k (the energy's own power of two, so that seeds far below the float
// range stay floats; the streaming kernels scale it to the slab) -- the
// reference's expressions in FP64 (src/energeticParticles.c:2300-2350),
// rounded to float once per call: the FP32 streaming kernels read them
// instead of spending FP64 pipe time on them at every launch.
__global__ void k_stream2_coef(RunView r) {
  const size_t total = (size_t)r.S * r.E * r.N;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const int il = (int)(i % r.N);
    const size_t se = i / r.N;
    const int e = (int)(se % r.E);
    const int s = (int)(se / r.E);
    const int L = r.list_size[s];
    float4 out = make_float4(0.f, 0.f, 0.f, 0.f);
    if (il < L) {
      const EnergyConsts ec = r.ec[e];
      const double dtMin = 0.4 * r.ds_min[s] * ec.vgrid_i;
      const double nst = floor(r.dt / dtMin + 1.0);
      const double dtProp = r.dt / (1.0 * (nst >= 1.0 ? nst : 1.0));
      const double dtProp_i = 1.0 / dtProp;
      const size_t sN = (size_t)s * r.N;
      const size_t gidx = sN + r.list[sN + il];
      const double tau = ec.vgrid_i * (ec.rig_lamo * r.mfp_node[gidx]);
      const double dsi = r.ds_i[sN + il];
      const double mult = (dtProp > tau) ? dsi * tau * dtProp_i : dsi * 1.0;
      // split form: the relaxation runs in the node phase instead
      const double emt = r.relax_in_stream ? exp(-dtProp / tau) : 1.0;
      // the relaxation weight om = 1 - exp(-dtProp/tau) as its multiple of
      // 2^-24 below (y: the fraction left over, z: that multiple): see
      // relax_weight
      const double om = (1.0 - emt) * 16777216.0;
      const double lo = floor(om);
      out = make_float4((float)mult, (float)(om - lo), (float)(lo * 0x1p-24),
                        (float)ldexp(seed_value(r, ec, r.seed_radial[gidx]), ec.seed_k));
    }
    r.scoef[i] = out;
  }
}

// seedPopulationCheck (src/energeticParticlesBoundary.c:28-59) alone, for
// runs without parallel diffusion, in the FP32 form: one thread per row,
// compared in FP64 true values, and the row renormalised (the seed may lie
// far above the row's values).
__global__ void k_seed_check32(RunView r) {
  const size_t items = (size_t)r.S * r.N * r.E;
  for (size_t it = blockIdx.x * (size_t)blockDim.x + threadIdx.x; it < items;
       it += (size_t)gridDim.x * blockDim.x) {
    const size_t g = it / r.E;
    const int e = (int)(it - g * r.E);
    const double seed = seed_value(r, r.ec[e], r.seed_radial[g]);
    float *fp = reinterpret_cast<float *>(r.f) + it * r.M;
    const int x = r.fexp[it];
    double mx = seed;
    for (int m = 0; m < r.M; ++m) mx = fmax(mx, ldexp((double)fp[m], -x));
    const int xn = row_exp_for(ilogb(mx));
    for (int m = 0; m < r.M; ++m) {
      double v = ldexp((double)fp[m], -x);
      if (v < seed) v = seed;
      const float w = (float)ldexp(v, xn);
      fp[m] = w < FLT_MIN ? FLT_MIN : w;
    }
    r.fexp[it] = (short)xn;
  }
}

int launch_seed_check32(const RunView &r, cudaStream_t st, uint64_t *launches) {
  const size_t items = (size_t)r.S * r.N * r.E;
  size_t b = (items + 255) / 256;
  if (b > 152 * 32) b = 152 * 32;
  k_seed_check32<<<(unsigned)b, 256, 0, st>>>(r);
  *launches += 1;
  return cudaGetLastError() == cudaSuccess ? 0 : EPREM_GPU_ERR_CUDA;
}

int launch_stream2_coef(const RunView &r, cudaStream_t st, uint64_t *launches) {
  const size_t total = (size_t)r.S * r.E * r.N;
  size_t b = (total + 255) / 256;
  if (b > 152 * 64) b = 152 * 64;
  k_stream2_coef<<<(unsigned)b, 256, 0, st>>>(r);
  *launches += 1;
  return cudaGetLastError() == cudaSuccess ? 0 : EPREM_GPU_ERR_CUDA;
}

namespace {
struct S2Shape {
  int mmax, T, npt;
};
// The mirrored kinds' own bin: M = 20 exactly (the CPU-runnable case's size,
// which the packed kinds run in the 24 bin with run-time guards), with shapes
// for short streams: 64 x 7 holds a 400-node stream in two warps.
#define EPREM_S2M20_SHAPES(X) X(20, 64, 7) X(20, 128, 8) X(20, 256, 4)
constexpr S2Shape kS2Shapes[] = {
#define EPREM_S2_ROW(MM, TT, NN) {MM, TT, NN},
    EPREM_S2_SHAPES(EPREM_S2_ROW) EPREM_S2M20_SHAPES(EPREM_S2_ROW)
#undef EPREM_S2_ROW
};
}  // namespace

// The shapes the mirrored kinds are built for: three of the 40 bin and the 20
// bin.  At N = 1500 the 128 x 4 shape in clusters of 3 (two CTAs of
// different slabs share an SM) took 14.8 ms per 96-stream launch, 256 x 3 in
// clusters of 2 19.4 ms.  Wider CTAs do not pay: the register file is split between the four
// warp schedulers, so 9 to 12 warps cap a thread at 168 registers, and 3 or 4
// list nodes of 40 cells then spill (288x4, 352x3, 384x3 measured with ptxas).
#define EPREM_S2M_SHAPES(X) X(40, 256, 4) X(40, 128, 4) X(40, 256, 3) EPREM_S2M20_SHAPES(X)

// shape: 0 automatic, k >= 1 the k-th shape of the mu bin.  Automatic: the
// bin's default when one CTA holds the stream, else the shape whose cluster
// wastes the fewest list-node slots (ties to the earlier shape).  The
// mirrored kinds need N + NPT - 1 slots (list node 0 may start up to NPT - 1
// slots in) and take only the shapes they are built for.
int plan_stream2(int N, int M, int m0, bool packed, bool filled, int mirror, bool bc, int shape,
                 StreamPlan *plan) {
  int mmax = 0;
  if (mirror) {  // their own bins: M exactly, halves of equal length
    if (!(packed && filled && bc) || !(M == 20 || M == 40) || 2 * m0 != M)
      return EPREM_GPU_ERR_ARG;
    mmax = M;
  }
  for (int b : {8, 16, 24, 32, 40, 48, 64})
    if (!mmax && M <= b && m0 <= b / 2 && M - m0 <= b / 2) { mmax = b; break; }
  if (!mmax) return EPREM_GPU_ERR_ARG;
  // packed: odd halves take one padding cell (mmax/2 is even, so it fits)
  if (filled && !(M == mmax && 2 * m0 == mmax)) return EPREM_GPU_ERR_ARG;
  const S2Shape *pick = nullptr;
  int k = 0;
  double best = 0.0;
  for (const S2Shape &sh : kS2Shapes) {
    if (sh.mmax != mmax) continue;
    ++k;
    bool built = !mirror;
#define EPREM_S2M_HAS(MM, TT, NN) built |= sh.mmax == MM && sh.T == TT && sh.npt == NN;
    EPREM_S2M_SHAPES(EPREM_S2M_HAS)
#undef EPREM_S2M_HAS
    if (!built) continue;
    const int per = sh.T * sh.npt, need = mirror ? N + sh.npt - 1 : N;
    const int cl = (need + per - 1) / per;
    if (cl > 8) continue;
    if (shape) {
      if (k == shape) pick = &sh;
      continue;
    }
    if (k == 1 && cl == 1) { pick = &sh; break; }
    const double use = (double)N / ((double)cl * per);
    if (!pick || use > best + 1e-9) { pick = &sh; best = use; }
  }
  if (!pick) return EPREM_GPU_ERR_ARG;
  plan->mmax = mmax;
  plan->threads = pick->T;
  plan->npt = pick->npt;
  plan->reg_coef = 2;  // marks the several-nodes-per-thread kernels
  plan->packed = packed ? 1 : 0;
  plan->filled = filled ? 1 : 0;
  plan->mirror = mirror;
  const int per = pick->T * pick->npt;
  plan->cluster = ((mirror ? N + pick->npt - 1 : N) + per - 1) / per;
  return 0;
}

// Shapes of M's bin: the larger count of the packed kinds' bin and, for M = 20,
// the mirrored kinds' own bin.
int stream2_shape_count(int M) {
  int mmax = 0;
  for (int b : {8, 16, 24, 32, 40, 48, 64})
    if (M <= b) { mmax = b; break; }
  int k = 0, k20 = 0;
  for (const S2Shape &sh : kS2Shapes) {
    k += sh.mmax == mmax;
    k20 += M == 20 && sh.mmax == 20;
  }
  return k > k20 ? k : k20;
}

static cudaError_t launch_cluster(const void *kern, dim3 grid, int T, int cluster, size_t dyn,
                                  cudaStream_t st, void **args) {
  if (dyn > 48 * 1024) {
    const cudaError_t e =
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
    if (e != cudaSuccess) return e;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
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
  return cudaLaunchKernelExC(&cfg, kern, args);
}

template <int MMAX, int T, int NPT>
static cudaError_t launch_stream2_t(const RunView &r, const StreamPlan &pl, int m0,
                                    cudaStream_t st) {
  constexpr size_t dyn = stream2_smem_bytes<MMAX, T>();
  void (*kern)(RunView, int) = !pl.packed  ? k_stream2<MMAX, T, NPT>
                               : pl.filled ? k_stream2_pairs<MMAX, T, NPT, true>
                                           : k_stream2_pairs<MMAX, T, NPT, false>;
  RunView rv = r;
  void *args[] = {&rv, &m0};
  return launch_cluster((const void *)kern, dim3(pl.cluster, r.S, r.E), T, pl.cluster, dyn, st,
                        args);
}

// The mirrored kernel of a plan: kind 7 with its coefficients in shared
// memory and, on one CTA per slab, the neighbour-warp halo hand-over; kind 6
// with the coefficients formed on the loop and a barrier per sub-cycle.
template <int MMAX, int T, int NPT, typename Args>
static cudaError_t launch_mirror_kind(const StreamPlan &pl, dim3 grid, Args args, bool multi,
                                      cudaStream_t st) {
  const void *kern;
  size_t dyn;
  if (pl.mirror == 2 && pl.cluster == 1) {
    kern = multi ? (const void *)k_stream2_mirror_multi<MMAX, T, NPT, true, 1>
                 : (const void *)k_stream2_mirror<MMAX, T, NPT, true, 1>;
    dyn = stream2_mirror_smem_bytes<MMAX, T, NPT, true>();
  } else if (pl.mirror == 2) {
    kern = multi ? (const void *)k_stream2_mirror_multi<MMAX, T, NPT, true, 0>
                 : (const void *)k_stream2_mirror<MMAX, T, NPT, true, 0>;
    dyn = stream2_mirror_smem_bytes<MMAX, T, NPT, true>();
  } else {
    kern = multi ? (const void *)k_stream2_mirror_multi<MMAX, T, NPT, false, 0>
                 : (const void *)k_stream2_mirror<MMAX, T, NPT, false, 0>;
    dyn = stream2_mirror_smem_bytes<MMAX, T, NPT, false>();
  }
  return launch_cluster(kern, grid, T, pl.cluster, dyn, st, args);
}

template <int MMAX, int T, int NPT>
static cudaError_t launch_stream2_mirror_t(const RunView &r, const StreamPlan &pl,
                                           cudaStream_t st) {
  RunView rv = r;
  int unused = 0;
  void *args[] = {&rv, &unused};
  return launch_mirror_kind<MMAX, T, NPT>(pl, dim3(pl.cluster, r.S, r.E), args, false, st);
}

template <int MMAX, int T, int NPT>
static cudaError_t launch_stream2_mirror_multi_t(const StreamPlan &pl, const MultiRunViews &mv,
                                                 const int4 *items, int n_items,
                                                 cudaStream_t st) {
  void *args[] = {const_cast<MultiRunViews *>(&mv), &items};
  return launch_mirror_kind<MMAX, T, NPT>(pl, dim3(pl.cluster * n_items, 1, 1), args, true, st);
}

template <int MMAX, int T, int NPT>
static cudaError_t launch_stream2_multi_t(const StreamPlan &pl, const MultiRunViews &mv,
                                          const int4 *items, int n_items, cudaStream_t st) {
  constexpr size_t dyn = stream2_smem_bytes<MMAX, T>();
  void (*kern)(const MultiRunViews, const int4 *) =
      pl.filled ? k_stream2_pairs_multi<MMAX, T, NPT, true>
                : k_stream2_pairs_multi<MMAX, T, NPT, false>;
  void *args[] = {const_cast<MultiRunViews *>(&mv), &items};
  return launch_cluster((const void *)kern, dim3(pl.cluster * n_items, 1, 1), T, pl.cluster, dyn,
                        st, args);
}

int launch_stream2_multi(const StreamPlan &pl, const MultiRunViews &mv, const int4 *items,
                         int n_items, cudaStream_t st, uint64_t *launches) {
  if (!pl.packed || n_items <= 0) return EPREM_GPU_ERR_ARG;
  cudaError_t err = cudaErrorInvalidValue;
  if (pl.mirror) {
#define EPREM_S2M_MCASE(MM, TT, NN)                                                \
  if (pl.mmax == MM && pl.threads == TT && pl.npt == NN)                           \
    err = launch_stream2_mirror_multi_t<MM, TT, NN>(pl, mv, items, n_items, st); \
  else
    EPREM_S2M_SHAPES(EPREM_S2M_MCASE) {}
#undef EPREM_S2M_MCASE
  } else {
#define EPREM_S2_MCASE(MM, TT, NN)                                          \
  if (pl.mmax == MM && pl.threads == TT && pl.npt == NN)                    \
    err = launch_stream2_multi_t<MM, TT, NN>(pl, mv, items, n_items, st); \
  else
    EPREM_S2_SHAPES(EPREM_S2_MCASE) {}
#undef EPREM_S2_MCASE
  }
  *launches += 1;
  return err == cudaSuccess ? 0 : EPREM_GPU_ERR_CUDA;
}

int launch_stream2(const RunView &r, const StreamPlan &pl, int m0, cudaStream_t st,
                   uint64_t *launches) {
  cudaError_t err = cudaErrorInvalidValue;
  if (pl.mirror) {
    if (!r.use_bc) return EPREM_GPU_ERR_ARG;  // the mirrored kinds need the seed boundary
#define EPREM_S2M_CASE(MM, TT, NN)                                \
  if (pl.mmax == MM && pl.threads == TT && pl.npt == NN)          \
    err = launch_stream2_mirror_t<MM, TT, NN>(r, pl, st);         \
  else
    EPREM_S2M_SHAPES(EPREM_S2M_CASE) {}
#undef EPREM_S2M_CASE
  } else {
#define EPREM_S2_CASE(MM, TT, NN)                                   \
  if (pl.mmax == MM && pl.threads == TT && pl.npt == NN)            \
    err = launch_stream2_t<MM, TT, NN>(r, pl, m0, st);             \
  else
    EPREM_S2_SHAPES(EPREM_S2_CASE) {}
#undef EPREM_S2_CASE
  }
  *launches += 1;
  return err == cudaSuccess ? 0 : EPREM_GPU_ERR_CUDA;
}

}  // namespace eprem
