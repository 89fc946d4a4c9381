// stream.cu -- streaming along each stream with isotropisation (K1).
//
// Restates DiffuseStreamData (src/energeticParticles.c:2240-2490) for one
// (stream, energy) slab per thread-block cluster:
//   * thread i of the cluster owns list node i (GetStreamList order) and keeps
//     all of that node's mu cells in registers for every sub-cycle;
//   * the upwind neighbour (list node i-1 for mu >= 0, i+1 for mu < 0) comes
//     from a warp shuffle; at warp edges from a small shared-memory edge
//     buffer, and at CTA edges from the neighbouring CTA's edge buffer through
//     distributed shared memory -- one cluster barrier per sub-cycle;
//   * the isotropisation mean over mu is a register sum in the owning thread.
// seedPopulationCheck (src/energeticParticlesBoundary.c:28-59) is applied as
// the slab is loaded; the thinned-out nodes receive their reference node's
// values on write-back, as the reference's shellRef copy does (:2448-2455).
#include <cooperative_groups.h>

#include "common.cuh"
#include "kernels.h"

namespace cg = cooperative_groups;

namespace eprem {

template <typename Real, int MMAX> struct StreamShape;
// Threads per CTA so that MMAX register slots per thread fit the SM's 64 K
// registers with one CTA per SM.
#define EPREM_STREAM_SHAPE(R, MM, TT) \
  template <> struct StreamShape<R, MM> { static constexpr int T = TT; };
EPREM_STREAM_SHAPE(double, 8, 1024)
EPREM_STREAM_SHAPE(double, 16, 768)
EPREM_STREAM_SHAPE(double, 24, 640)
EPREM_STREAM_SHAPE(double, 32, 512)
EPREM_STREAM_SHAPE(double, 40, 512)
EPREM_STREAM_SHAPE(double, 48, 384)
EPREM_STREAM_SHAPE(double, 64, 256)
EPREM_STREAM_SHAPE(float, 8, 1024)
EPREM_STREAM_SHAPE(float, 16, 1024)
EPREM_STREAM_SHAPE(float, 24, 1024)
EPREM_STREAM_SHAPE(float, 32, 768)
EPREM_STREAM_SHAPE(float, 40, 768)
EPREM_STREAM_SHAPE(float, 48, 640)
EPREM_STREAM_SHAPE(float, 64, 512)
#undef EPREM_STREAM_SHAPE

template <typename Real, int MMAX, int T>
__global__ void __launch_bounds__(T, 1) k_stream(RunView r, int m0) {
  constexpr int W = T / 32;
  constexpr unsigned FULL = 0xffffffffu;
  __shared__ Real edge[2 * 2 * W * MMAX];  // [parity][hi=lane31 / lo=lane0][warp][mu]
  __shared__ Real del_s[MMAX];
  cg::cluster_group cluster = cg::this_cluster();
  const int C = (int)cluster.num_blocks();
  const int crank = (int)cluster.block_rank();
  const int s = blockIdx.y;
  const int e = r.E - 1 - (int)blockIdx.z;  // most sub-cycles first
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int M = r.M, N = r.N;
  const int L = r.list_size[s];
  if (L < 3) return;  // flagged by the geometry pass; uniform over the cluster

  const EnergyConsts ec = r.ec[e];
  const double dtMin = 0.4 * r.ds_min[s] * ec.vgrid_i;
  const double nst = floor(r.dt / dtMin + 1.0);
  if (!(nst <= (double)r.max_subcycles)) {
    if (crank == 0 && tid == 0) set_error(r.status, EPREM_GPU_ERR_SUBCYCLES, 1, s, -1, e, -1);
    return;  // uniform over the cluster
  }
  const int nsteps = (int)nst;
  const double dtProp = r.dt / (1.0 * nsteps);
  const double dtProp_i = 1.0 / dtProp;
  if (crank == 0 && tid == 0) {
    atomicMax(&r.status->max_stream, nsteps);
    atomicAdd(&r.status->stream_cs, (unsigned long long)nsteps * L * M);
  }
  for (int mu = tid; mu < M; mu += T) del_s[mu] = (Real)(ec.vgrid * dtProp * r.mugrid[mu]);

  const int i = crank * T + tid;
  const bool active = i < L;
  const bool first = (i == 0), last = (i == L - 1);
  const size_t sN = (size_t)s * N;
  Real fr[MMAX];
#pragma unroll
  for (int mu = 0; mu < MMAX; ++mu) fr[mu] = (Real)0;
  double mult = 0.0, emt = 0.0;
  Real bcv = (Real)0;
  bool bc_node = false;
  int k = 0;
  if (active) {
    k = r.list[sN + i];
    const size_t gidx = sN + k;
    const double tau = ec.vgrid_i * (ec.rig_lamo * r.mfp_node[gidx]);
    const double dsi = r.ds_i[sN + i];
    mult = (dtProp > tau) ? dsi * tau * dtProp_i : dsi * 1.0;
    emt = exp(-dtProp / tau);
    const double seedv = seed_value(r, ec, r.seed_radial[gidx]);
    const Real *fp = reinterpret_cast<const Real *>(r.f) + (gidx * r.E + e) * M;
#pragma unroll
    for (int mu = 0; mu < MMAX; ++mu) {
      if (mu < M) {
        Real v = fp[mu];
        if (r.check_seed && (double)v < seedv) v = to_real<Real>(seedv);
        fr[mu] = v;
      }
    }
    if (r.use_bc && i < 3) {
      bc_node = true;
      bcv = to_real<Real>(seedv);
    }
  }
  const Real c_mult = (Real)mult;
  const Real c_emt = (Real)emt;
  const Real c_omemt = (Real)(1.0 - emt);
  const Real inv_m = (Real)(1.0 / M);
  const Real *prev_edge = crank > 0 ? cluster.map_shared_rank(edge, crank - 1) : nullptr;
  const Real *next_edge = crank < C - 1 ? cluster.map_shared_rank(edge, crank + 1) : nullptr;
  __syncthreads();

  for (int step = 0; step < nsteps; ++step) {
    const int p = step & 1;
    Real *ep = edge + p * 2 * W * MMAX;
    if (bc_node) {
#pragma unroll
      for (int mu = 0; mu < MMAX; ++mu) fr[mu] = bcv;
    }
    if (lane == 31) {
#pragma unroll
      for (int mu = 0; mu < MMAX; ++mu)
        if (mu < M) ep[warp * MMAX + mu] = fr[mu];
    }
    if (lane == 0) {
#pragma unroll
      for (int mu = 0; mu < MMAX; ++mu)
        if (mu < M) ep[(W + warp) * MMAX + mu] = fr[mu];
    }
    if (C > 1)
      cluster.sync();
    else
      __syncthreads();
    Real acc = (Real)0;
#pragma unroll
    for (int mu = 0; mu < MMAX; ++mu) {
      if (mu < M) {
        const Real c = c_mult * del_s[mu];
        Real fn;
        if (mu >= m0) {  // mugrid[mu] >= 0: upwind from list node i-1
          Real nb = __shfl_up_sync(FULL, fr[mu], 1);
          if (lane == 0) {
            if (warp > 0)
              nb = ep[(warp - 1) * MMAX + mu];
            else if (prev_edge)
              nb = prev_edge[p * 2 * W * MMAX + (W - 1) * MMAX + mu];
          }
          fn = first ? fr[mu] : fr[mu] + c * (nb - fr[mu]);
        } else {  // mu < 0: upwind from list node i+1
          Real nb = __shfl_down_sync(FULL, fr[mu], 1);
          if (lane == 31) {
            if (warp < W - 1)
              nb = ep[(W + warp + 1) * MMAX + mu];
            else if (next_edge)
              nb = next_edge[p * 2 * W * MMAX + W * MMAX + mu];
          }
          fn = last ? fr[mu] : fr[mu] + c * (fr[mu] - nb);
        }
        fr[mu] = fn;
        acc += fn;
      }
    }
    // f = iso + (f_new - iso) exp(-dt/tau), iso = mean over mu
    const Real iso_part = (inv_m * acc) * c_omemt;
#pragma unroll
    for (int mu = 0; mu < MMAX; ++mu)
      if (mu < M) fr[mu] = fr[mu] * c_emt + iso_part;
  }

  if (active) {
    int code = 0;
    const Real fl = Floor<Real>::v();
#pragma unroll
    for (int mu = 0; mu < MMAX; ++mu) {
      if (mu < M) {
        Real v = fr[mu];
        if (bad_value(v, &code)) set_error(r.status, code, 1, s, k, e, mu);
        fr[mu] = v < fl ? fl : v;
      }
    }
    // node k and the thinned nodes that reference it (previous list node + 1 .. k)
    const int kfirst = first ? 0 : r.list[sN + i - 1] + 1;
    for (int kk = kfirst; kk <= k; ++kk) {
      Real *op = reinterpret_cast<Real *>(r.f) + ((sN + kk) * r.E + e) * M;
#pragma unroll
      for (int mu = 0; mu < MMAX; ++mu)
        if (mu < M) op[mu] = fr[mu];
    }
  }
  if (C > 1) cluster.sync();  // neighbours may still read this CTA's edge buffer
}

// seedPopulationCheck alone, for runs without parallel diffusion.
template <typename Real>
__global__ void k_seed_check(RunView r) {
  const size_t items = (size_t)r.S * r.N * r.E;
  for (size_t it = blockIdx.x * (size_t)blockDim.x + threadIdx.x; it < items;
       it += (size_t)gridDim.x * blockDim.x) {
    const size_t gidx = it / r.E;
    const int e = (int)(it % r.E);
    const double seedv = seed_value(r, r.ec[e], r.seed_radial[gidx]);
    Real *fp = reinterpret_cast<Real *>(r.f) + it * r.M;
    for (int mu = 0; mu < r.M; ++mu)
      if ((double)fp[mu] < seedv) fp[mu] = to_real<Real>(seedv);
  }
}

static const int kStreamBins[] = {8, 16, 24, 32, 40, 48, 64};

static int stream_threads(int precision, int mmax) {
  if (precision == EPREM_FP64) {
    switch (mmax) {
      case 8: return StreamShape<double, 8>::T;
      case 16: return StreamShape<double, 16>::T;
      case 24: return StreamShape<double, 24>::T;
      case 32: return StreamShape<double, 32>::T;
      case 40: return StreamShape<double, 40>::T;
      case 48: return StreamShape<double, 48>::T;
      default: return StreamShape<double, 64>::T;
    }
  }
  switch (mmax) {
    case 8: return StreamShape<float, 8>::T;
    case 16: return StreamShape<float, 16>::T;
    case 24: return StreamShape<float, 24>::T;
    case 32: return StreamShape<float, 32>::T;
    case 40: return StreamShape<float, 40>::T;
    case 48: return StreamShape<float, 48>::T;
    default: return StreamShape<float, 64>::T;
  }
}

int plan_stream(int precision, int N, int M, StreamPlan *plan) {
  int mmax = 0;
  for (int b : kStreamBins)
    if (M <= b) { mmax = b; break; }
  if (!mmax) return EPREM_GPU_ERR_ARG;
  plan->mmax = mmax;
  plan->threads = stream_threads(precision, mmax);
  plan->cluster = (N + plan->threads - 1) / plan->threads;
  if (plan->cluster > 8) return EPREM_GPU_ERR_ARG;  // portable cluster limit
  return 0;
}

template <typename Real, int MMAX>
static cudaError_t launch_stream_t(const RunView &r, int cluster, int m0, cudaStream_t st) {
  constexpr int T = StreamShape<Real, MMAX>::T;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(cluster, r.S, r.E);
  cfg.blockDim = dim3(T, 1, 1);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = cluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k_stream<Real, MMAX, T>, r, m0);
}

template <typename Real>
static cudaError_t dispatch_stream(const RunView &r, const StreamPlan &pl, int m0,
                                   cudaStream_t st) {
  switch (pl.mmax) {
    case 8: return launch_stream_t<Real, 8>(r, pl.cluster, m0, st);
    case 16: return launch_stream_t<Real, 16>(r, pl.cluster, m0, st);
    case 24: return launch_stream_t<Real, 24>(r, pl.cluster, m0, st);
    case 32: return launch_stream_t<Real, 32>(r, pl.cluster, m0, st);
    case 40: return launch_stream_t<Real, 40>(r, pl.cluster, m0, st);
    case 48: return launch_stream_t<Real, 48>(r, pl.cluster, m0, st);
    default: return launch_stream_t<Real, 64>(r, pl.cluster, m0, st);
  }
}

int launch_stream(const RunView &r, const StreamPlan &plan, int m0, cudaStream_t st,
                  uint64_t *launches) {
  cudaError_t err = r.precision == EPREM_FP64 ? dispatch_stream<double>(r, plan, m0, st)
                                              : dispatch_stream<float>(r, plan, m0, st);
  *launches += 1;
  return err == cudaSuccess ? 0 : EPREM_GPU_ERR_CUDA;
}

int launch_seed_check(const RunView &r, cudaStream_t st, uint64_t *launches) {
  const size_t items = (size_t)r.S * r.N * r.E;
  int blocks = (int)((items + 255) / 256);
  if (blocks > 152 * 32) blocks = 152 * 32;
  if (r.precision == EPREM_FP64)
    k_seed_check<double><<<blocks, 256, 0, st>>>(r);
  else
    k_seed_check<float><<<blocks, 256, 0, st>>>(r);
  *launches += 1;
  return cudaGetLastError() == cudaSuccess ? 0 : EPREM_GPU_ERR_CUDA;
}

}  // namespace eprem
