// geometry.cu -- per-call stream geometry (K0).
//
// Node positions do not change inside updateEnergeticParticles (the driver
// moves nodes before calling it, src/eprem.c:620-671), so the reference's
// per-sub-step recomputation of these quantities yields the same values every
// sub-step; they are computed once per call here:
//   * updateStreamValues (src/simCore.c:326-435): ds, mhdBmagPlus/Minus;
//   * the node factors of sepSeedFunction and meanFreePath;
//   * min_tau over nodes >= 1 (src/energeticParticles.c:149-156);
//   * GetStreamList + FindSegmentLengths (src/energeticParticles.c:2150-2234,
//     :2496-2601): thinned list, 1/ds of list segments, dsMin per stream.
#include "common.cuh"
#include "kernels.h"

namespace eprem {

// |d| summed x, y, z in that order without fused multiply-adds, so that ds,
// dsMin and therefore the sub-cycle counts match the reference bit for bit.
__device__ __forceinline__ double dist3(double dx, double dy, double dz) {
  return sqrt(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
}

__global__ void k_node_prep(RunView r, double norm_radius, double neg_beta, int mfp_type,
                            double mfp_power, double bs_au) {
  const size_t SN = (size_t)r.S * r.N;
  for (size_t g = blockIdx.x * (size_t)blockDim.x + threadIdx.x; g < SN;
       g += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(g % r.N);
    const double rs = r.r_scale;
    const double *rx = node_field(r, EPREM_NODE_RX), *ry = node_field(r, EPREM_NODE_RY),
                 *rz = node_field(r, EPREM_NODE_RZ), *bmag = node_field(r, EPREM_NODE_BMAG);
    // __dmul_rn keeps the scaled coordinates out of fused multiply-adds with
    // the differences below (the reference scales, then subtracts).
    double x = __dmul_rn(rx[g], rs), y = __dmul_rn(ry[g], rs), z = __dmul_rn(rz[g], rs);
    double ds, bminus, bplus;
    if (k == 0) {
      double px = __dmul_rn(rx[g + 1], rs), py = __dmul_rn(ry[g + 1], rs),
             pz = __dmul_rn(rz[g + 1], rs);
      ds = dist3(px - x, py - y, pz - z);
      bminus = bmag[g];
      bplus = bmag[g + 1];
    } else if (k == r.N - 1) {
      double mx = __dmul_rn(rx[g - 1], rs), my = __dmul_rn(ry[g - 1], rs),
             mz = __dmul_rn(rz[g - 1], rs);
      ds = dist3(x - mx, y - my, z - mz);
      bminus = bmag[g - 1];
      bplus = bmag[g];
    } else {
      double px = __dmul_rn(rx[g + 1], rs), py = __dmul_rn(ry[g + 1], rs),
             pz = __dmul_rn(rz[g + 1], rs);
      double mx = __dmul_rn(rx[g - 1], rs), my = __dmul_rn(ry[g - 1], rs),
             mz = __dmul_rn(rz[g - 1], rs);
      double dsp = dist3(px - x, py - y, pz - z);
      double dsm = dist3(x - mx, y - my, z - mz);
      ds = 0.5 * (dsp + dsm);
      bminus = bmag[g - 1];
      bplus = bmag[g + 1];
    }
    node_field(r, EPREM_NODE_DS)[g] = ds;
    node_field(r, EPREM_NODE_BMAG_MINUS)[g] = bminus;
    node_field(r, EPREM_NODE_BMAG_PLUS)[g] = bplus;
    const double rmag = node_field(r, EPREM_NODE_RMAG)[g];
    // radialTerm of sepSeedFunction (src/energeticParticlesBoundary.c:100)
    r.seed_radial[g] = pow(rmag / norm_radius, neg_beta);
    // pow factor of meanFreePathR / meanFreePathB (src/meanFreePath.c:13-27)
    double mf = (mfp_type == 2) ? pow(bs_au / bmag[g], mfp_power) : pow(rmag * rs, mfp_power);
    r.mfp_node[g] = mf;
    if (k >= 1) {
      double tmin = DBL_MAX;
      for (int e = 0; e < r.E; e++) {
        double tau = r.ec[e].rig_lamo * mf * r.ec[e].vgrid_i;
        if (tau < tmin) tmin = tau;
      }
      atomic_min_pos(&r.status->min_tau_bits, tmin);
    }
  }
}

// One warp per stream.  Lane 0 runs the order-dependent thinning scan over
// positions staged in shared memory; the warp then forms the segment lengths.
__global__ void k_stream_list(RunView r) {
  extern __shared__ double sh[];
  const int s = blockIdx.x;
  const int N = r.N, lane = threadIdx.x;
  double *xs = sh, *ys = sh + N, *zs = sh + 2 * N;
  int *lst = reinterpret_cast<int *>(sh + 3 * N);
  __shared__ int Lsh;
  const size_t base = (size_t)s * N;
  const double rs = r.r_scale;
  const double *rx = node_field(r, EPREM_NODE_RX), *ry = node_field(r, EPREM_NODE_RY),
               *rz = node_field(r, EPREM_NODE_RZ);
  for (int k = lane; k < N; k += 32) {
    xs[k] = __dmul_rn(rx[base + k], rs);
    ys[k] = __dmul_rn(ry[base + k], rs);
    zs[k] = __dmul_rn(rz[base + k], rs);
  }
  __syncwarp();
  if (lane == 0) {
    int L = 0, down = 0, up;
    for (int sh_i = 0; sh_i < N; sh_i++) {
      if (sh_i < N - 1) {
        up = sh_i + 1;
      } else {
        up = sh_i;
        down = sh_i - 1;
      }
      double dsh = dist3(xs[up] - xs[down], ys[up] - ys[down], zs[up] - zs[down]);
      if ((dsh > r.dsh_min) || (sh_i == N - 1)) {
        lst[L++] = sh_i;
        down = sh_i + 1;
      }
    }
    Lsh = L;
  }
  __syncwarp();
  const int L = Lsh;
  if (L < 3) {
    if (lane == 0) {
      set_error(r, EPREM_GPU_ERR_STATE, 4, s, L, -1, -1);
      r.list_size[s] = L;
    }
    return;
  }
  double dmin = 10000.0 * rs;
  for (int sl = lane; sl < L; sl += 32) {
    const int th = lst[sl];
    double ds_sl;
    if (sl == 0) {
      int nx = lst[1];
      ds_sl = dist3(xs[nx] - xs[th], ys[nx] - ys[th], zs[nx] - zs[th]);
      dmin = fmin(dmin, ds_sl);
    } else if (sl == L - 1) {
      int pv = lst[sl - 1];
      ds_sl = dist3(xs[th] - xs[pv], ys[th] - ys[pv], zs[th] - zs[pv]);
      dmin = fmin(dmin, ds_sl);
    } else {
      int nx = lst[sl + 1], pv = lst[sl - 1];
      double ds1 = dist3(xs[nx] - xs[th], ys[nx] - ys[th], zs[nx] - zs[th]);
      double ds9 = dist3(xs[th] - xs[pv], ys[th] - ys[pv], zs[th] - zs[pv]);
      dmin = fmin(dmin, fmin(ds1, ds9));
      ds_sl = 0.5 * (ds1 + ds9);
    }
    r.list[base + sl] = th;
    r.ds_i[base + sl] = 1.0 / ds_sl;
  }
  for (int o = 16; o > 0; o >>= 1) dmin = fmin(dmin, __shfl_xor_sync(0xffffffffu, dmin, o));
  if (lane == 0) {
    r.list_size[s] = L;
    r.ds_min[s] = dmin;
    if (!(dmin > 0.0)) set_error(r, EPREM_GPU_ERR_DS, 4, s, -1, -1, -1);
  }
}

int launch_geometry(const RunView &r, cudaStream_t st, double norm_radius, double neg_beta,
                    int mfp_type, double mfp_power, double bs_au, uint64_t *launches) {
  const size_t SN = (size_t)r.S * r.N;
  int blocks = (int)((SN + 255) / 256);
  if (blocks > 152 * 32) blocks = 152 * 32;
  k_node_prep<<<blocks, 256, 0, st>>>(r, norm_radius, neg_beta, mfp_type, mfp_power, bs_au);
  size_t smem = (size_t)r.N * (3 * sizeof(double) + sizeof(int));
  // per launch: runs of different sizes share the kernel's attribute
  if (cudaFuncSetAttribute(k_stream_list, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem) != cudaSuccess)
    return EPREM_GPU_ERR_CUDA;
  k_stream_list<<<r.S, 32, smem, st>>>(r);
  *launches += 2;
  return cudaGetLastError() == cudaSuccess ? 0 : EPREM_GPU_ERR_CUDA;
}

int geometry_smem_bytes(int N) { return N * (3 * (int)sizeof(double) + (int)sizeof(int)); }

int setup_geometry_attrs(int N) {
  int smem = geometry_smem_bytes(N);
  if (cudaFuncSetAttribute(k_stream_list, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) !=
      cudaSuccess)
    return EPREM_GPU_ERR_CUDA;
  return 0;
}

}  // namespace eprem
