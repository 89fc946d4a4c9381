// mas.cu -- MAS background on the nodes (A12) and the RK4 node push (A13).
//
//   k_mas_update_mhd : updateMhd's MHD_MAS branch (src/flow.c:36-154) with
//                      masGetNode (src/masInterp.c:31-68): masTriLinear
//                      (:539-740: per field a binary search on each of its
//                      three staggered meshes in both time slots, trilinear
//                      interpolation, blend by s_cor, unit conversion, Vr
//                      floor) inside masRadialMax, masWind (:1007-1065)
//                      beyond it;
//   k_mas_move_nodes : masMoveNodes (:1344-1393), RK4 through vMas
//                      (:1281-1296) and sphToCartVector (src/geometry.c:89-121).
// One thread per node, FP64 arithmetic on FP32 field data, as the reference.
// All time slices the caller loads stay resident in HBM; a step selects two.
#include "common.cuh"
#include "kernels.h"

namespace eprem {

constexpr double kRsun = 6.96e10;
constexpr double kRsAu = kRsun / kAu;
constexpr double kMasLengthNorm = 6.96e10;
constexpr double kMasTimeNorm = 1445.87003080685;
constexpr double kMasRhoNorm = 1.6726e-16;

struct MasNodeVals {
  double br, bt, bp, vr, vt, vp, d;
};

// masTriLinearBinarySearch (src/masInterp.c:118-171)
__device__ __forceinline__ double mas_search(const float *A, double key, int *imin, int *imax,
                                             int lower, int upper) {
  while (upper != (lower + 1)) {
    const int imid = (lower + upper) / 2;
    if (A[imid] < key)
      lower = imid;
    else
      upper = imid;
  }
  *imin = lower;
  *imax = upper;
  if (A[lower] > key) return 0.0;
  if (A[upper] < key) return 1.0;
  return (key - A[lower]) / (A[upper] - A[lower]);
}

// masInterpolate (src/masInterp.c:178-200), data [phi][theta][r]
__device__ __forceinline__ double mas_interp(const float *V, int r0, int r1, int t0, int t1,
                                             int p0, int p1, double rd, double td, double pd,
                                             int rDim, int tDim) {
  auto ix = [&](int r, int t, int p) {
    return (size_t)r + (size_t)rDim * t + (size_t)rDim * tDim * p;
  };
  const double c00 = V[ix(r0, t0, p0)] * (1.0 - rd) + V[ix(r1, t0, p0)] * rd;
  const double c10 = V[ix(r0, t0, p1)] * (1.0 - rd) + V[ix(r1, t0, p1)] * rd;
  const double c01 = V[ix(r0, t1, p0)] * (1.0 - rd) + V[ix(r1, t1, p0)] * rd;
  const double c11 = V[ix(r0, t1, p1)] * (1.0 - rd) + V[ix(r1, t1, p1)] * rd;
  const double c0 = c00 * (1.0 - pd) + c10 * pd;
  const double c1 = c01 * (1.0 - pd) + c11 * pd;
  return c0 * (1.0 - td) + c1 * td;
}

__device__ double mas_field(const MasView &mv, int f, double rr, double th, double ph) {
  double val[2];
#pragma unroll
  for (int sl = 0; sl < 2; sl++) {
    const MasSlotDev &S = sl ? mv.s1 : mv.s0;
    int r0, r1, t0, t1, p0, p1;
    const double rd = mas_search(S.mesh[f][0], rr, &r0, &r1, 0, S.dims[f][0] - 1);
    const double td = mas_search(S.mesh[f][1], th, &t0, &t1, 0, S.dims[f][1] - 1);
    const double pd = mas_search(S.mesh[f][2], ph, &p0, &p1, 0, S.dims[f][2] - 1);
    val[sl] = mas_interp(S.data[f], r0, r1, t0, t1, p0, p1, rd, td, pd, S.dims[f][0],
                         S.dims[f][1]);
  }
  return (1.0 - mv.s_cor) * val[0] + mv.s_cor * val[1];
}

// masTriLinear (src/masInterp.c:539-740); position r in AU.
__device__ void mas_trilinear(const MasView &mv, double pr, double pth, double pph,
                              MasNodeVals *o) {
  const double rr = pr / kRsAu;
  double ph = pph - mv.phi_offset;
  while (ph < 0.0) ph += 2.0 * kPi;
  while (ph > 2.0 * kPi) ph -= 2.0 * kPi;
  const double mhd_b_norm = sqrt(kMp * kMhdDensityNorm) * kC;
  const double bconv = sqrt(4.0 * kPi * kMasRhoNorm);
  o->bp = mas_field(mv, 0, rr, pth, ph) * bconv * kMasLengthNorm / kMasTimeNorm / mhd_b_norm;
  o->bt = mas_field(mv, 1, rr, pth, ph) * bconv * kMasLengthNorm / kMasTimeNorm / mhd_b_norm;
  o->br = mas_field(mv, 2, rr, pth, ph) * bconv * kMasLengthNorm / kMasTimeNorm / mhd_b_norm;
  o->vp = mas_field(mv, 3, rr, pth, ph) * (kMasLengthNorm / kMasTimeNorm) / kC;
  o->vt = mas_field(mv, 4, rr, pth, ph) * (kMasLengthNorm / kMasTimeNorm) / kC;
  o->vr = mas_field(mv, 5, rr, pth, ph) * (kMasLengthNorm / kMasTimeNorm) / kC;
  if (o->vr < mv.v_min / kC) o->vr = mv.v_min / kC;
  o->d = mas_field(mv, 6, rr, pth, ph) * (kMasRhoNorm / kMp) / kMhdDensityNorm;
}

// masWind (src/masInterp.c:1007-1065) from node g's previous values.
__device__ void mas_wind(const RunView &r, const MasView &mv, size_t g, MasNodeVals *o) {
  auto F = [&](int field) { return node_field(r, field)[g]; };
  const double ox = F(EPREM_NODE_ROLD_X), oy = F(EPREM_NODE_ROLD_Y), oz = F(EPREM_NODE_ROLD_Z);
  const double br = F(EPREM_NODE_BR), bt = F(EPREM_NODE_BTHETA), bp = F(EPREM_NODE_BPHI);
  const double vr = F(EPREM_NODE_VR), vt = F(EPREM_NODE_VTHETA), vp = F(EPREM_NODE_VPHI);
  const double rho = F(EPREM_NODE_DENSITY);
  const double rOldmag = sqrt(ox * ox + oy * oy + oz * oz);
  const double rmag = F(EPREM_NODE_RMAG);
  const double q = rOldmag / rmag;
  o->br = br * q * q;
  o->bt = bt * q;
  o->bp = bp * q;
  if (mv.cor_rotate_fake > 0 && mv.rotate_solution > 0) {
    const double theta = acos(F(EPREM_NODE_RZ) / rmag);
    const double thetaOld = acos(oz / rOldmag);
    o->bp += (mv.r_scale * mv.omega_sun / vr) *
             (rOldmag * br * sin(thetaOld) - rmag * o->br * sin(theta));
  }
  o->vr = vr;
  o->vt = vt * q;
  o->vp = vp * q;
  o->d = rho * q * q;
}

// cartToSphPosAu (src/geometry.c:131-157)
__device__ __forceinline__ void sph_au(double rs, double x, double y, double z, double *pr,
                                       double *pth, double *pph) {
  const double ax = x * rs, ay = y * rs, az = z * rs;
  *pr = sqrt(ax * ax + ay * ay + az * az);
  *pth = acos(az / *pr);
  double ph = atan2(ay, ax);
  while (ph < 0.0) ph += 2.0 * kPi;
  while (ph > 2.0 * kPi) ph -= 2.0 * kPi;
  *pph = ph;
}

__device__ __forceinline__ void mas_get_node(const RunView &r, const MasView &mv, size_t g,
                                             double pr, double pth, double pph, MasNodeVals *o) {
  if (pr <= mv.radial_max * kRsAu)
    mas_trilinear(mv, pr, pth, pph, o);
  else
    mas_wind(r, mv, g, o);
}

__global__ void k_mas_update_mhd(RunView r, MasView mv, double t_del) {
  const size_t SN = (size_t)r.S * r.N;
  for (size_t g = blockIdx.x * (size_t)blockDim.x + threadIdx.x; g < SN;
       g += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(g % r.N);
    auto F = [&](int field) -> double & { return node_field(r, field)[g]; };
    F(EPREM_NODE_BMAG_OLD) = F(EPREM_NODE_BMAG);
    F(EPREM_NODE_DENSITY_OLD) = F(EPREM_NODE_DENSITY);
    F(EPREM_NODE_VSPH_OLD_R) = F(EPREM_NODE_VR);
    F(EPREM_NODE_VSPH_OLD_THETA) = F(EPREM_NODE_VTHETA);
    F(EPREM_NODE_VSPH_OLD_PHI) = F(EPREM_NODE_VPHI);
    F(EPREM_NODE_DS_OLD) = F(EPREM_NODE_DS);
    F(EPREM_NODE_ROLDER_X) = F(EPREM_NODE_RX);
    F(EPREM_NODE_ROLDER_Y) = F(EPREM_NODE_RY);
    F(EPREM_NODE_ROLDER_Z) = F(EPREM_NODE_RZ);
    const double x = F(EPREM_NODE_RX), y = F(EPREM_NODE_RY), z = F(EPREM_NODE_RZ);
    const double rmag = F(EPREM_NODE_RMAG);
    double pr, pth, pph;
    sph_au(r.r_scale, x, y, z, &pr, &pth, &pph);
    MasNodeVals mn;
    mas_get_node(r, mv, g, pr, pth, pph, &mn);
    const double dens = mn.d;
    F(EPREM_NODE_DENSITY) = dens;
    F(EPREM_NODE_DIVV) = (dens <= 0.0) ? 0.0 : -1.0 * log(dens / F(EPREM_NODE_DENSITY_OLD)) / t_del;
    const double theta = acos(z / rmag), phi = atan2(y, x);
    const double st = sin(theta), ct = cos(theta), sp = sin(phi), cp = cos(phi);
    const double Vr = mn.vr, Vt = mn.vt, Vp = mn.vp;
    F(EPREM_NODE_VR) = Vr;
    F(EPREM_NODE_VTHETA) = Vt;
    F(EPREM_NODE_VPHI) = Vp;
    F(EPREM_NODE_VMAG) = sqrt(Vr * Vr + Vt * Vt + Vp * Vp);
    F(EPREM_NODE_VVEC_X) = Vr * st * cp + Vt * ct * cp - Vp * sp;
    F(EPREM_NODE_VVEC_Y) = Vr * st * sp + Vt * ct * sp + Vp * cp;
    F(EPREM_NODE_VVEC_Z) = Vr * ct - Vt * st;
    const double Br = mn.br, Bt = mn.bt, Bp = mn.bp;
    F(EPREM_NODE_BR) = Br;
    F(EPREM_NODE_BTHETA) = Bt;
    F(EPREM_NODE_BPHI) = Bp;
    const double Bmag = sqrt(Br * Br + Bt * Bt + Bp * Bp);
    F(EPREM_NODE_BMAG) = Bmag;
    F(EPREM_NODE_BVEC_X) = Br * st * cp + Bt * ct * cp - Bp * sp;
    F(EPREM_NODE_BVEC_Y) = Br * st * sp + Bt * ct * sp + Bp * cp;
    F(EPREM_NODE_BVEC_Z) = Br * ct - Bt * st;
    if (k == 0) {
      F(EPREM_NODE_DUPAR) = 0.0;
      F(EPREM_NODE_DLNB) = 0.0;
      F(EPREM_NODE_DLNN) = 0.0;
    } else {
      const double dupar = (Vr - F(EPREM_NODE_VSPH_OLD_R)) * Br +
                           (Vt - F(EPREM_NODE_VSPH_OLD_THETA)) * Bt +
                           (Vp - F(EPREM_NODE_VSPH_OLD_PHI)) * Bp;
      F(EPREM_NODE_DUPAR) = dupar / Bmag;
      F(EPREM_NODE_DLNB) = log(Bmag / F(EPREM_NODE_BMAG_OLD));
      F(EPREM_NODE_DLNN) = log(dens / F(EPREM_NODE_DENSITY_OLD));
    }
  }
}

// sphToCartVector (src/geometry.c:89-121)
__device__ __forceinline__ void sph_to_cart(double vr, double vt, double vp, double x, double y,
                                            double z, double *ox, double *oy, double *oz) {
  const double rmag = sqrt(x * x + y * y + z * z);
  const double rho = sqrt(rmag * rmag - z * z);
  if ((rmag - fabs(z)) < kVerySmall) {
    *ox = 0.0;
    *oy = 0.0;
  } else {
    *ox = x / rmag * vr + x * z / (rmag * rho) * vt - y / rho * vp;
    *oy = y / rmag * vr + y * z / (rmag * rho) * vt + x / rho * vp;
  }
  *oz = z / rmag * vr - rho / rmag * vt;
}

__device__ __forceinline__ void vmas(const RunView &r, const MasView &mv, size_t g, double x,
                                     double y, double z, double *vx, double *vy, double *vz) {
  double pr, pth, pph;
  sph_au(r.r_scale, x, y, z, &pr, &pth, &pph);
  MasNodeVals mn;
  mas_get_node(r, mv, g, pr, pth, pph, &mn);
  sph_to_cart(mn.vr, mn.vt, mn.vp, x, y, z, vx, vy, vz);
}

__global__ void k_mas_move_nodes(RunView r, MasView mv, double dt) {
  const size_t SN = (size_t)r.S * r.N;
  for (size_t g = blockIdx.x * (size_t)blockDim.x + threadIdx.x; g < SN;
       g += (size_t)gridDim.x * blockDim.x) {
    if (g % r.N == 0) continue;  // the innermost node stays on the inner boundary
    double *rx = node_field(r, EPREM_NODE_RX), *ry = node_field(r, EPREM_NODE_RY),
           *rz = node_field(r, EPREM_NODE_RZ);
    const double x0 = rx[g], y0 = ry[g], z0 = rz[g];
    const double h = dt / r.r_scale;
    double vx, vy, vz;
    vmas(r, mv, g, x0, y0, z0, &vx, &vy, &vz);
    const double k1x = vx * h, k1y = vy * h, k1z = vz * h;
    vmas(r, mv, g, x0 + k1x * 0.5, y0 + k1y * 0.5, z0 + k1z * 0.5, &vx, &vy, &vz);
    const double k2x = vx * h, k2y = vy * h, k2z = vz * h;
    vmas(r, mv, g, x0 + k2x * 0.5, y0 + k2y * 0.5, z0 + k2z * 0.5, &vx, &vy, &vz);
    const double k3x = vx * h, k3y = vy * h, k3z = vz * h;
    vmas(r, mv, g, x0 + k3x, y0 + k3y, z0 + k3z, &vx, &vy, &vz);
    const double k4x = vx * h, k4y = vy * h, k4z = vz * h;
    const double sixth = 1.0 / 6.0;
    const double x1 = x0 + sixth * (k1x + 2.0 * k2x + 2.0 * k3x + k4x);
    const double y1 = y0 + sixth * (k1y + 2.0 * k2y + 2.0 * k3y + k4y);
    const double z1 = z0 + sixth * (k1z + 2.0 * k2z + 2.0 * k3z + k4z);
    node_field(r, EPREM_NODE_ROLD_X)[g] = x0;
    node_field(r, EPREM_NODE_ROLD_Y)[g] = y0;
    node_field(r, EPREM_NODE_ROLD_Z)[g] = z0;
    rx[g] = x1;
    ry[g] = y1;
    rz[g] = z1;
    node_field(r, EPREM_NODE_RMAG)[g] = sqrt((x1 * x1) + (y1 * y1) + (z1 * z1));
  }
}

static int mas_grid(size_t n) {
  size_t b = (n + 127) / 128;
  return (int)(b > 152 * 64 ? 152 * 64 : (b ? b : 1));
}

int launch_mas_update_mhd(const RunView &r, const MasView &mv, double t_del, cudaStream_t st,
                          uint64_t *launches) {
  k_mas_update_mhd<<<mas_grid((size_t)r.S * r.N), 128, 0, st>>>(r, mv, t_del);
  *launches += 1;
  return cudaGetLastError() == cudaSuccess ? 0 : EPREM_GPU_ERR_CUDA;
}

int launch_mas_move_nodes(const RunView &r, const MasView &mv, double dt, cudaStream_t st,
                          uint64_t *launches) {
  k_mas_move_nodes<<<mas_grid((size_t)r.S * r.N), 128, 0, st>>>(r, mv, dt);
  *launches += 1;
  return cudaGetLastError() == cudaSuccess ? 0 : EPREM_GPU_ERR_CUDA;
}

}  // namespace eprem
