// stream.cu -- streaming along each stream with isotropisation (K1).
//
// Restates DiffuseStreamData (src/energeticParticles.c:2240-2490) for one
// (stream, energy) slab per CTA or thread-block cluster:
//   * thread i owns list node i (GetStreamList order) and keeps that node's mu
//     cells in registers for all of the slab's sub-cycles;
//   * the upwind neighbour (list node i-1 for mu >= 0, i+1 for mu < 0) comes
//     from a warp shuffle; lanes at warp edges read a halo slot in their own
//     CTA's shared memory, which the neighbouring warp -- or, across a CTA
//     edge, the neighbouring CTA of the cluster, by a distributed-shared-memory
//     store -- fills before the sub-cycle's barrier.  The inner loop therefore
//     only ever loads from local shared memory;
//   * the isotropisation mean over mu is a register sum in the owning thread.
// The upwind coefficients mult*del_fac are fixed for the slab and held in
// shared memory (the FP64 form is bound by the FP64 pipe, next to which
// shared-memory loads cost nothing).  This is the plain FP64 form's kernel;
// the FP32 form streams with stream2.cu.
// seedPopulationCheck (src/energeticParticlesBoundary.c:28-59) is applied as
// the slab is loaded; thinned-out nodes receive their reference node's values
// on write-back, as the reference's shellRef copy does (:2448-2455).
#include <cooperative_groups.h>

#include "common.cuh"
#include "kernels.h"

namespace cg = cooperative_groups;

namespace eprem {

// Threads per CTA (multiples of 128, the register-allocation granule).
template <typename Real, int MMAX, bool RegCoef> struct StreamShape;
#define EPREM_STREAM_SHAPE(R, MM, RC, TT) \
  template <> struct StreamShape<R, MM, RC> { static constexpr int T = TT; };
EPREM_STREAM_SHAPE(double, 8, false, 1024)
EPREM_STREAM_SHAPE(double, 16, false, 768)
EPREM_STREAM_SHAPE(double, 24, false, 512)
EPREM_STREAM_SHAPE(double, 32, false, 512)
EPREM_STREAM_SHAPE(double, 40, false, 512)
EPREM_STREAM_SHAPE(double, 48, false, 384)
EPREM_STREAM_SHAPE(double, 64, false, 384)
#undef EPREM_STREAM_SHAPE

// Shared memory of one CTA: coefficient table (shared-coefficient shapes) and
// the halo slots.
template <typename Real, int MMAX, bool RegCoef>
constexpr size_t stream_smem_bytes() {
  constexpr int T = StreamShape<Real, MMAX, RegCoef>::T;
  constexpr int W = T / 32;
  return (RegCoef ? 0 : sizeof(Real) * MMAX * T) + sizeof(Real) * 2 * 2 * (W + 1) * MMAX;
}

template <typename Real, int MMAX, bool RegCoef>
__global__ void __launch_bounds__((StreamShape<Real, MMAX, RegCoef>::T), 1)
    k_stream(RunView r, int m0) {
  constexpr int T = StreamShape<Real, MMAX, RegCoef>::T;
  constexpr int W = T / 32;
  constexpr unsigned FULL = 0xffffffffu;
  // halo slots, double-buffered by sub-cycle parity p:
  //   hi[p][w][mu], w = 0..W : slot w+1 holds lane 31 of warp w; slot 0 the
  //                            previous CTA's last lane (written remotely);
  //   lo[p][w][mu], w = 0..W : slot w holds lane 0 of warp w; slot W the next
  //                            CTA's first lane (written remotely).
  extern __shared__ __align__(16) unsigned char sm_raw[];
  Real *coef = reinterpret_cast<Real *>(sm_raw);  // [mu][T], shared-coefficient shapes
  Real *halo = coef + (RegCoef ? 0 : MMAX * T);
  auto hi = [&](int p, int w) { return halo + ((p * 2 + 0) * (W + 1) + w) * MMAX; };
  auto lo = [&](int p, int w) { return halo + ((p * 2 + 1) * (W + 1) + w) * MMAX; };

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
    if (crank == 0 && tid == 0) set_error(r, EPREM_GPU_ERR_SUBCYCLES, 1, s, -1, e, -1);
    return;  // uniform over the cluster
  }
  const int nsteps = (int)nst;
  const double dtProp = r.dt / (1.0 * nsteps);
  const double dtProp_i = 1.0 / dtProp;
  if (crank == 0 && tid == 0) {
    atomicMax(&r.status->max_stream, nsteps);
    atomicAdd(&r.status->stream_cs, (unsigned long long)nsteps * L * M);
  }
  // zero the halo slots: the ones no neighbour writes stay zero (finite)
  for (int j = tid; j < 2 * 2 * (W + 1) * MMAX; j += T) halo[j] = (Real)0;

  const int i = crank * T + tid;
  const bool active = i < L;
  const size_t sN = (size_t)s * N;
  Real fr[MMAX], cf[RegCoef ? MMAX : 1];
#pragma unroll
  for (int mu = 0; mu < MMAX; ++mu) {
    fr[mu] = (Real)0;
    if (RegCoef) cf[mu] = (Real)0;
    else if (mu < M) coef[mu * T + tid] = (Real)0;
  }
  double emt = 0.0;
  Real bcv = (Real)0;
  bool bc_node = false;
  int k = 0;
  if (active) {
    k = r.list[sN + i];
    const size_t gidx = sN + k;
    const double tau = ec.vgrid_i * (ec.rig_lamo * r.mfp_node[gidx]);
    const double dsi = r.ds_i[sN + i];
    const double mult = (dtProp > tau) ? dsi * tau * dtProp_i : dsi * 1.0;
    emt = r.relax_in_stream ? exp(-dtProp / tau) : 1.0;  // split form: node phase relaxes
    const double seedv = seed_value(r, ec, r.seed_radial[gidx]);
    const Real *fp = reinterpret_cast<const Real *>(r.f) + (gidx * r.E + e) * M;
#pragma unroll
    for (int mu = 0; mu < MMAX; ++mu) {
      if (mu < M) {
        Real v = fp[mu];
        if (r.check_seed && (double)v < seedv) v = to_real<Real>(seedv);
        fr[mu] = v;
        // upwind coefficient mult * del_fac (src/energeticParticles.c:2346, :2386);
        // zero where the reference copies the cell unchanged (the first list
        // node for mu >= 0, the last for mu < 0, :2381 and :2393)
        const bool edge_cell = (mu >= m0) ? (i == 0) : (i == L - 1);
        const double del_fac = ec.vgrid * dtProp * r.mugrid[mu];
        const Real c = edge_cell ? (Real)0 : (Real)(mult * del_fac);
        if (RegCoef)
          cf[mu] = c;
        else
          coef[mu * T + tid] = c;
      }
    }
    if (r.use_bc && i < 3) {
      bc_node = true;
      bcv = to_real<Real>(seedv);
    }
  }
  const Real c_emt = (Real)emt;
  const Real c_omemt = (Real)(1.0 - emt);
  const Real inv_m = (Real)(1.0 / M);
  // remote halo slots this CTA fills in its neighbours
  Real *next_hi0 = (C > 1 && crank < C - 1) ? cluster.map_shared_rank(halo, crank + 1) : nullptr;
  Real *prev_loW = (C > 1 && crank > 0) ? cluster.map_shared_rank(halo, crank - 1) : nullptr;
  if (C > 1)
    cluster.sync();  // halo zeroing above is complete before any remote store lands
  else
    __syncthreads();

  for (int step = 0; step < nsteps; ++step) {
    const int p = step & 1;
    if (bc_node) {
#pragma unroll
      for (int mu = 0; mu < MMAX; ++mu) fr[mu] = bcv;
    }
    if (lane == 31) {
      Real *dst = hi(p, warp + 1);
      Real *rdst = (warp == W - 1 && next_hi0)
                       ? next_hi0 + ((p * 2 + 0) * (W + 1) + 0) * MMAX : nullptr;
#pragma unroll
      for (int mu = 0; mu < MMAX; ++mu)
        if (mu < M) {
          dst[mu] = fr[mu];
          if (rdst) rdst[mu] = fr[mu];
        }
    }
    if (lane == 0) {
      Real *dst = lo(p, warp);
      Real *rdst = (warp == 0 && prev_loW)
                       ? prev_loW + ((p * 2 + 1) * (W + 1) + W) * MMAX : nullptr;
#pragma unroll
      for (int mu = 0; mu < MMAX; ++mu)
        if (mu < M) {
          dst[mu] = fr[mu];
          if (rdst) rdst[mu] = fr[mu];
        }
    }
    if (C > 1)
      cluster.sync();
    else
      __syncthreads();
    const Real *my_hi = hi(p, warp);      // lane 31 of warp-1 / previous CTA
    const Real *my_lo = lo(p, warp + 1);  // lane 0 of warp+1 / next CTA
    Real acc = (Real)0;
#pragma unroll
    for (int mu = 0; mu < MMAX; ++mu) {
      if (mu < M) {
        const Real c = RegCoef ? cf[mu] : coef[mu * T + tid];
        Real fn;
        if (mu >= m0) {  // mugrid[mu] >= 0: upwind from list node i-1
          Real nb = __shfl_up_sync(FULL, fr[mu], 1);
          if (lane == 0) nb = my_hi[mu];
          fn = fr[mu] + c * (nb - fr[mu]);
        } else {  // mu < 0: upwind from list node i+1
          Real nb = __shfl_down_sync(FULL, fr[mu], 1);
          if (lane == 31) nb = my_lo[mu];
          fn = fr[mu] + c * (fr[mu] - nb);
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
        if (bad_value(v, &code)) set_error(r, code, 1, s, k, e, mu);
        fr[mu] = v < fl ? fl : v;
      }
    }
    // node k and the thinned nodes that reference it (previous list node + 1 .. k)
    const int kfirst = (i == 0) ? 0 : r.list[sN + i - 1] + 1;
    for (int kk = kfirst; kk <= k; ++kk) {
      Real *op = reinterpret_cast<Real *>(r.f) + ((sN + kk) * r.E + e) * M;
#pragma unroll
      for (int mu = 0; mu < MMAX; ++mu)
        if (mu < M) op[mu] = fr[mu];
    }
  }
  if (C > 1) cluster.sync();  // no CTA leaves while a neighbour may still store into it
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

template <typename Real, bool RC>
static int threads_for(int mmax) {
  switch (mmax) {
    case 8: return StreamShape<Real, 8, RC>::T;
    case 16: return StreamShape<Real, 16, RC>::T;
    case 24: return StreamShape<Real, 24, RC>::T;
    case 32: return StreamShape<Real, 32, RC>::T;
    case 40: return StreamShape<Real, 40, RC>::T;
    case 48: return StreamShape<Real, 48, RC>::T;
    default: return StreamShape<Real, 64, RC>::T;
  }
}

// variant = kind + 8 * shape.  kind 0 automatic; FP32 form (stream2.cu):
// 3 several list nodes per thread, 4 the same with packed fp32x2 arithmetic
// (an odd mu half padded with a zero cell), 5 as 4 with the cell guards
// resolved at compile time (M fills its bin, m0 = M/2), 6 and 7 as 5 with the
// mu < 0 half in mirror order, one upwind coefficient per two cells (6 formed
// on the sub-cycle loop, 7 from shared memory; both need the seed boundary)
// -- the automatic kind is the first of 7, 5, 4, 3 that fits; shape 0 lets
// plan_stream2 choose the CTA shape from N, k >= 1 names the k-th shape of
// the mu bin.  The FP64 form has one shape (k_stream, coefficients in shared
// memory); variants 1 and 2 name it there.
int plan_stream(int precision, int N, int M, int m0, int variant, bool bc, StreamPlan *plan) {
  if (precision == EPREM_FP32) {
    const int kind = variant % 8, shape = variant / 8;
    if (variant < 0 || kind == 1 || kind == 2) return EPREM_GPU_ERR_ARG;
    if (kind == 6) return plan_stream2(N, M, m0, true, true, 1, bc, shape, plan);
    if ((kind == 0 || kind == 7) && plan_stream2(N, M, m0, true, true, 2, bc, shape, plan) == 0)
      return 0;
    if (kind == 7) return EPREM_GPU_ERR_ARG;
    if ((kind == 0 || kind == 5) && plan_stream2(N, M, m0, true, true, 0, bc, shape, plan) == 0)
      return 0;
    if ((kind == 0 || kind == 4) && plan_stream2(N, M, m0, true, false, 0, bc, shape, plan) == 0)
      return 0;
    if ((kind == 0 || kind == 3) && plan_stream2(N, M, m0, false, false, 0, bc, shape, plan) == 0)
      return 0;
    return EPREM_GPU_ERR_ARG;
  }
  if (variant > 2) return EPREM_GPU_ERR_ARG;
  int mmax = 0;
  for (int b : kStreamBins)
    if (M <= b) { mmax = b; break; }
  if (!mmax) return EPREM_GPU_ERR_ARG;
  plan->mmax = mmax;
  plan->reg_coef = 0;
  plan->mirror = 0;
  plan->threads = threads_for<double, false>(mmax);
  plan->cluster = (N + plan->threads - 1) / plan->threads;
  if (plan->cluster > 8) return EPREM_GPU_ERR_ARG;  // portable cluster limit
  return 0;
}

template <typename Real, int MMAX, bool RC>
static cudaError_t launch_stream_t(const RunView &r, int cluster, int m0, cudaStream_t st) {
  constexpr int T = StreamShape<Real, MMAX, RC>::T;
  constexpr size_t dyn = stream_smem_bytes<Real, MMAX, RC>();
  auto kern = k_stream<Real, MMAX, RC>;
  cudaError_t e =
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
  if (e != cudaSuccess) return e;
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

template <typename Real, bool RC>
static cudaError_t dispatch_mmax(const RunView &r, const StreamPlan &pl, int m0,
                                 cudaStream_t st) {
  switch (pl.mmax) {
    case 8: return launch_stream_t<Real, 8, RC>(r, pl.cluster, m0, st);
    case 16: return launch_stream_t<Real, 16, RC>(r, pl.cluster, m0, st);
    case 24: return launch_stream_t<Real, 24, RC>(r, pl.cluster, m0, st);
    case 32: return launch_stream_t<Real, 32, RC>(r, pl.cluster, m0, st);
    case 40: return launch_stream_t<Real, 40, RC>(r, pl.cluster, m0, st);
    case 48: return launch_stream_t<Real, 48, RC>(r, pl.cluster, m0, st);
    default: return launch_stream_t<Real, 64, RC>(r, pl.cluster, m0, st);
  }
}

int launch_stream(const RunView &r, const StreamPlan &plan, int m0, cudaStream_t st,
                  uint64_t *launches) {
  if (plan.reg_coef == 2) return launch_stream2(r, plan, m0, st, launches);
  if (r.precision != EPREM_FP64) return EPREM_GPU_ERR_ARG;
  const cudaError_t err = dispatch_mmax<double, false>(r, plan, m0, st);
  *launches += 1;
  return err == cudaSuccess ? 0 : EPREM_GPU_ERR_CUDA;
}

int launch_seed_check(const RunView &r, cudaStream_t st, uint64_t *launches) {
  if (r.precision == EPREM_FP32) return launch_seed_check32(r, st, launches);
  const size_t items = (size_t)r.S * r.N * r.E;
  int blocks = (int)((items + 255) / 256);
  if (blocks > 152 * 32) blocks = 152 * 32;
  k_seed_check<double><<<blocks, 256, 0, st>>>(r);
  *launches += 1;
  return cudaGetLastError() == cudaSuccess ? 0 : EPREM_GPU_ERR_CUDA;
}

}  // namespace eprem
