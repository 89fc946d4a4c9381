// mhd.cu -- analytic MHD background on the nodes, node advection, flux,
// and the host-format conversions of f.
//
//   k_update_mhd : updateMhd for mhdGridStatus == MHD_DEFAULT
//                  (src/flow.c:36-154 with mhdDensity :241-275, mhdV :356-403,
//                  mhdB :281-350, idealShockFactor :623-651,
//                  cartToSphPosAu src/geometry.c:131-150)
//   k_move_nodes : moveNodes (src/simCore.c:737-785) with the MHD_DEFAULT
//                  branch of delrFlow (src/flow.c:162-196)
//   k_omni_flux  : computeFlux without its unit scale (src/unifiedOutput.c:153-180)
// All FP64, one thread per node.
#include "common.cuh"
#include "kernels.h"

namespace eprem {

__device__ double shock_factor(const MhdParams &p, double r, double tg) {
  const double front = (p.speed / kC) * (tg - p.init_time / kDay) + p.r_scale;
  const double exponent = exp(2.0 * (p.sharp / p.scale_len) * (r - front));
  double ratio;
  if (exponent >= 1.0e8)
    ratio = 1.0;
  else if (exponent <= 1.0e-8)
    ratio = -1.0;
  else
    ratio = (exponent - 1.0) / (exponent + 1.0);
  const double factor = (1.0 + ((1.0 - ratio) * 0.5 * (p.jump - 1.0)));
  const double falloff = exp(p.falloff * (r - front));
  return 1 + (factor - 1) * falloff;
}

// parkerB (src/flow.c:443-472) at (r AU, theta), ideal shock included.
__device__ void parker_b(const MhdParams &p, double r, double theta, double Vr, int isn,
                         double tg, double B[3]) {
  B[0] = p.mhd_bs_au / (r * r);
  B[1] = 0.0;
  B[2] = -1.0 * r * B[0] * (p.omega_sun / (Vr + kVerySmall)) * sin(theta);
  if (p.ideal_shock > 0 && isn > 0) {
    const double sf = shock_factor(p, r, tg);
    B[0] *= sf;
    B[1] *= sf;
    B[2] *= sf;
  }
}

// curlBoverB2 (src/flow.c:479-616): curl(B)/B^2 of the Parker field by
// centred differences at (r +- 0.001 AU, theta +- pi/100, phi +- pi/100),
// theta folded back into [0, pi]; the field has no phi dependence, so the
// phi offsets leave r and theta, and their differences vanish as there.
// Spherical components (r, theta, phi), the reference's operation order.
__device__ void curl_bover_b2(const MhdParams &p, double x, double y, double z, double Vr,
                              int isn, double tg, double curl[3]) {
  const double rcw = 0.001, tcw = kPi / 100.0, pcw = kPi / 100.0;
  const double rr = p.r_scale * sqrt(x * x + y * y + z * z);
  const double th = acos(z * p.r_scale / rr);
  const double rp = rr + rcw, rm = rr - rcw;
  double tp = th + tcw;
  if (tp > kPi) tp = 2.0 * kPi - tp;
  double tm = th - tcw;
  if (tm < 0.0) tm *= -1.0;
  double B_rm[3], B_rp[3], B_tm[3], B_tp[3], B_pc[3];
  parker_b(p, rm, th, Vr, isn, tg, B_rm);
  parker_b(p, rp, th, Vr, isn, tg, B_rp);
  parker_b(p, rr, tm, Vr, isn, tg, B_tm);
  parker_b(p, rr, tp, Vr, isn, tg, B_tp);
  parker_b(p, rr, th, Vr, isn, tg, B_pc);  // both phi offsets
  const double m_rm = sqrt(B_rm[0] * B_rm[0] + B_rm[1] * B_rm[1] + B_rm[2] * B_rm[2]);
  const double m_rp = sqrt(B_rp[0] * B_rp[0] + B_rp[1] * B_rp[1] + B_rp[2] * B_rp[2]);
  const double m_tm = sqrt(B_tm[0] * B_tm[0] + B_tm[1] * B_tm[1] + B_tm[2] * B_tm[2]);
  const double m_tp = sqrt(B_tp[0] * B_tp[0] + B_tp[1] * B_tp[1] + B_tp[2] * B_tp[2]);
  const double m_pc = sqrt(B_pc[0] * B_pc[0] + B_pc[1] * B_pc[1] + B_pc[2] * B_pc[2]);
  double A, B;
  A = (0.5 / tcw) * (B_tp[2] * sin(tp) / (m_tp * m_tp) - B_tm[2] * sin(tm) / (m_tm * m_tm));
  B = (0.5 / pcw) * (B_pc[1] / (m_pc * m_pc) - B_pc[1] / (m_pc * m_pc));
  curl[0] = (1.0 / (rr * sin(th))) * (A - B);
  A = (1.0 / sin(th)) * (0.5 / pcw) * (B_pc[0] / (m_pc * m_pc) - B_pc[0] / (m_pc * m_pc));
  B = (0.5 / rcw) * (rp * B_rp[2] / (m_rp * m_rp) - rm * B_rm[2] / (m_rm * m_rm));
  curl[1] = (1.0 / rr) * (A - B);
  A = (0.5 / rcw) * (rp * B_rp[1] / (m_rp * m_rp) - rm * B_rm[1] / (m_rm * m_rm));
  B = (0.5 / tcw) * (B_tp[0] / (m_tp * m_tp) - B_tm[0] / (m_tm * m_tm));
  curl[2] = (1.0 / rr) * (A - B);
}

// tg_dev, when given, holds the run's time on the device (graph replays of an
// ensemble step); tg is then the offset added to it.
__global__ void k_update_mhd(RunView r, MhdParams p, double tg, const double *tg_dev) {
  if (tg_dev) tg = *tg_dev + tg;
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
    int isn = 0;
    if (p.ideal_shock > 0) {
      const double ax = x * p.r_scale, ay = y * p.r_scale, az = z * p.r_scale;
      const double rr = sqrt(ax * ax + ay * ay + az * az);
      const double th = acos(az / rr);
      double ph = atan2(ay, ax);
      while (ph < 0.0) ph += (2.0 * kPi);
      if (rr <= p.speed * tg) {
        if (p.width == 0.0)
          isn = 1;
        else if ((fmin((2 * kPi) - fabs(ph - p.phi), fabs(ph - p.phi)) < (p.width / 2.0)) &&
                 (fabs(th - p.theta) < (p.width / 2.0)))
          isn = 1;
      }
    }
    const double rr = rmag * p.r_scale;
    double dens = p.mhd_ns_au / (rr * rr);
    if (p.ideal_shock > 0 && isn > 0) dens *= shock_factor(p, rr, tg);
    F(EPREM_NODE_DENSITY) = dens;
    F(EPREM_NODE_DIVV) = (dens <= 0.0) ? 0.0 : -1.0 * log(dens / F(EPREM_NODE_DENSITY_OLD)) / p.t_del;
    const double theta = acos(z / rmag);
    const double phi = atan2(y, x);
    const double st = sin(theta), ct = cos(theta), sp = sin(phi), cp = cos(phi);
    double Vr = p.mhd_us;
    if (p.ideal_shock > 0 && isn > 0) Vr *= shock_factor(p, rmag * p.r_scale, tg);
    const double Vt = 0.0, Vp = 0.0;
    F(EPREM_NODE_VR) = Vr;
    F(EPREM_NODE_VTHETA) = Vt;
    F(EPREM_NODE_VPHI) = Vp;
    F(EPREM_NODE_VMAG) = sqrt(Vr * Vr + Vt * Vt + Vp * Vp);
    F(EPREM_NODE_VVEC_X) = Vr * st * cp + Vt * ct * cp - Vp * sp;
    F(EPREM_NODE_VVEC_Y) = Vr * st * sp + Vt * ct * sp + Vp * cp;
    F(EPREM_NODE_VVEC_Z) = Vr * ct - Vt * st;
    const double Br = p.mhd_bs_au / (rr * rr);
    const double Bt = 0.0;
    const double Bp = -1.0 * rr * Br * (p.omega_sun / (Vr + kVerySmall)) * st;
    F(EPREM_NODE_BR) = Br;
    F(EPREM_NODE_BTHETA) = Bt;
    F(EPREM_NODE_BPHI) = Bp;
    const double Bmag = sqrt(Br * Br + Bt * Bt + Bp * Bp);
    F(EPREM_NODE_BMAG) = Bmag;
    F(EPREM_NODE_BVEC_X) = Br * st * cp + Bt * ct * cp - Bp * sp;
    F(EPREM_NODE_BVEC_Y) = Br * st * sp + Bt * ct * sp + Bp * cp;
    F(EPREM_NODE_BVEC_Z) = Br * ct - Bt * st;
    if (r.curl) {  // useDrift: mhdCurlBoverB2 (src/flow.c:127-128)
      double cv[3];
      curl_bover_b2(p, x, y, z, Vr, isn, tg, cv);
      for (int c = 0; c < 3; c++) r.curl[(size_t)c * r.node_stride + g] = cv[c];
    }
    if (k == 0) {  // rank-0 INNER_ACTIVE_SHELL (src/flow.c:131-137)
      F(EPREM_NODE_DUPAR) = 0.0;
      F(EPREM_NODE_DLNB) = 0.0;
      F(EPREM_NODE_DLNN) = 0.0;
    } else {
      double dupar = (Vr - F(EPREM_NODE_VSPH_OLD_R)) * Br +
                     (Vt - F(EPREM_NODE_VSPH_OLD_THETA)) * Bt +
                     (Vp - F(EPREM_NODE_VSPH_OLD_PHI)) * Bp;
      F(EPREM_NODE_DUPAR) = dupar / Bmag;
      F(EPREM_NODE_DLNB) = log(Bmag / F(EPREM_NODE_BMAG_OLD));
      F(EPREM_NODE_DLNN) = log(dens / F(EPREM_NODE_DENSITY_OLD));
    }
  }
}

__global__ void k_move_nodes(RunView r, double dt) {
  const size_t SN = (size_t)r.S * r.N;
  for (size_t g = blockIdx.x * (size_t)blockDim.x + threadIdx.x; g < SN;
       g += (size_t)gridDim.x * blockDim.x) {
    if (g % r.N == 0) continue;  // the innermost node stays on the inner boundary
    double *rx = node_field(r, EPREM_NODE_RX), *ry = node_field(r, EPREM_NODE_RY),
           *rz = node_field(r, EPREM_NODE_RZ);
    double x = rx[g], y = ry[g], z = rz[g];
    const double dx = dt * node_field(r, EPREM_NODE_VVEC_X)[g] / r.r_scale;
    const double dy = dt * node_field(r, EPREM_NODE_VVEC_Y)[g] / r.r_scale;
    const double dz = dt * node_field(r, EPREM_NODE_VVEC_Z)[g] / r.r_scale;
    node_field(r, EPREM_NODE_ROLD_X)[g] = x;
    node_field(r, EPREM_NODE_ROLD_Y)[g] = y;
    node_field(r, EPREM_NODE_ROLD_Z)[g] = z;
    x += dx;
    y += dy;
    z += dz;
    rx[g] = x;
    ry[g] = y;
    rz[g] = z;
    node_field(r, EPREM_NODE_RMAG)[g] = sqrt((x * x) + (y * y) + (z * z));
  }
}

template <typename Real>
__global__ void k_omni_flux(RunView r, double *out) {
  const size_t items = (size_t)r.S * r.N * r.E;
  for (size_t it = blockIdx.x * (size_t)blockDim.x + threadIdx.x; it < items;
       it += (size_t)gridDim.x * blockDim.x) {
    const Real *fp = reinterpret_cast<const Real *>(r.f) + it * r.M;
    double iso = 0.0;
    for (int m = 0; m < r.M; ++m) iso += (double)fp[m];
    iso /= r.M;
    if (sizeof(Real) == 4) iso = ldexp(iso, -(int)r.fexp[it]);  // the row's exponent
    out[it] = 2.0 * r.ec[it % r.E].egrid * iso;
  }
}

// FP64 rows (host values) <-> the FP32 form's rows with their exponents: a
// row's exponent brings its largest value to [2^kRowTop, 2^(kRowTop+1));
// scaling by a power of two is exact, so the float rounding is the plain one.
__global__ void k_rows_to_f32(const double *src, float *dst, short *xp, size_t nrows, int M) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < nrows;
       i += (size_t)gridDim.x * blockDim.x) {
    const double *a = src + i * M;
    double mx = 0.0;
    for (int m = 0; m < M; ++m) mx = fmax(mx, a[m]);
    const int x = mx > 0.0 ? row_exp_for(ilogb(mx)) : 0;
    float *b = dst + i * M;
    for (int m = 0; m < M; ++m) {
      const float v = (float)ldexp(a[m], x);
      b[m] = v < FLT_MIN ? FLT_MIN : v;
    }
    xp[i] = (short)x;
  }
}
__global__ void k_rows_to_f64(const float *src, const short *xp, double *dst, size_t nrows,
                              int M) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < nrows;
       i += (size_t)gridDim.x * blockDim.x) {
    const int x = xp[i];
    for (int m = 0; m < M; ++m) dst[i * M + m] = ldexp((double)src[i * M + m], -x);
  }
}

static int grid_for(size_t n) {
  size_t b = (n + 255) / 256;
  return (int)(b > 152 * 32 ? 152 * 32 : (b ? b : 1));
}

int launch_update_mhd(const RunView &r, const MhdParams &p, double tg, cudaStream_t st,
                      uint64_t *launches, const double *tg_dev) {
  k_update_mhd<<<grid_for((size_t)r.S * r.N), 256, 0, st>>>(r, p, tg, tg_dev);
  *launches += 1;
  return cudaGetLastError() == cudaSuccess ? 0 : EPREM_GPU_ERR_CUDA;
}

__global__ void k_advance_time(double *t, double dt) {
  if (threadIdx.x == 0) *t += dt;
}

int launch_advance_time(double *t_dev, double dt, cudaStream_t st, uint64_t *launches) {
  k_advance_time<<<1, 32, 0, st>>>(t_dev, dt);
  *launches += 1;
  return cudaGetLastError() == cudaSuccess ? 0 : EPREM_GPU_ERR_CUDA;
}

int launch_move_nodes(const RunView &r, double dt, cudaStream_t st, uint64_t *launches) {
  k_move_nodes<<<grid_for((size_t)r.S * r.N), 256, 0, st>>>(r, dt);
  *launches += 1;
  return cudaGetLastError() == cudaSuccess ? 0 : EPREM_GPU_ERR_CUDA;
}

int launch_omni_flux(const RunView &r, double *out, cudaStream_t st, uint64_t *launches) {
  const size_t items = (size_t)r.S * r.N * r.E;
  if (r.precision == EPREM_FP64)
    k_omni_flux<double><<<grid_for(items), 256, 0, st>>>(r, out);
  else
    k_omni_flux<float><<<grid_for(items), 256, 0, st>>>(r, out);
  *launches += 1;
  return cudaGetLastError() == cudaSuccess ? 0 : EPREM_GPU_ERR_CUDA;
}

// FP32 form: rows [row0, row0 + nrows) of the view between FP64 staging and
// the device's rows.  to_device: staging -> f; else f -> staging.
int launch_convert_f(const RunView &r, size_t row0, size_t nrows, double *stage, int to_device,
                     cudaStream_t st, uint64_t *launches) {
  float *f = reinterpret_cast<float *>(r.f) + row0 * r.M;
  short *xp = r.fexp + row0;
  if (to_device)
    k_rows_to_f32<<<grid_for(nrows), 256, 0, st>>>(stage, f, xp, nrows, r.M);
  else
    k_rows_to_f64<<<grid_for(nrows), 256, 0, st>>>(f, xp, stage, nrows, r.M);
  *launches += 1;
  return cudaGetLastError() == cudaSuccess ? 0 : EPREM_GPU_ERR_CUDA;
}

// rippleShellsOut (src/simCore.c:700-735) for f: node k of every stream takes
// node k-1's values (the outermost node's are dropped) and node 0 takes the
// stream's template row (the reference's INNER_SHELL).  A thread owns one
// (stream, energy, mu) cell and walks the nodes outward-in, reading a batch
// of nodes before writing them, so every value is read before it is
// overwritten; in the FP32 form the mu = 0 thread moves the row's exponent
// alike.  tmpl: S*E*M doubles; node 0's rows are written by k_ripple_rows.
template <typename Real>
__global__ void k_ripple_f(RunView r, const double *tmpl) {
  const size_t EM = (size_t)r.E * r.M;
  const size_t cells = (size_t)r.S * EM;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < cells;
       c += (size_t)gridDim.x * blockDim.x) {
    const size_t s = c / EM, j = c - s * EM;
    Real *p = reinterpret_cast<Real *>(r.f) + s * r.N * EM + j;
    const bool xrow = sizeof(Real) == 4 && j % r.M == 0;
    short *xp = xrow ? r.fexp + s * r.N * r.E + j / r.M : nullptr;
    for (int k = r.N - 1; k >= 1; k -= 8) {
      const int cnt = k < 8 ? k : 8;
      Real v[8];
      short x[8];
#pragma unroll
      for (int u = 0; u < 8; ++u)
        if (u < cnt) {
          v[u] = p[(size_t)(k - 1 - u) * EM];
          if (xrow) x[u] = xp[(size_t)(k - 1 - u) * r.E];
        }
#pragma unroll
      for (int u = 0; u < 8; ++u)
        if (u < cnt) {
          p[(size_t)(k - u) * EM] = v[u];
          if (xrow) xp[(size_t)(k - u) * r.E] = x[u];
        }
    }
    if (sizeof(Real) == 8) p[0] = (Real)tmpl[c];
  }
}

// Node 0's rows from the template (FP32 form), after k_ripple_f.
__global__ void k_ripple_rows(RunView r, const double *tmpl) {
  const size_t rows = (size_t)r.S * r.E;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < rows;
       i += (size_t)gridDim.x * blockDim.x) {
    const size_t s = i / r.E, e = i - s * r.E;
    const double *a = tmpl + i * r.M;
    double mx = 0.0;
    for (int m = 0; m < r.M; ++m) mx = fmax(mx, a[m]);
    const int x = mx > 0.0 ? row_exp_for(ilogb(mx)) : 0;
    float *b = reinterpret_cast<float *>(r.f) + (s * r.N * r.E + e) * r.M;
    for (int m = 0; m < r.M; ++m) {
      const float v = (float)ldexp(a[m], x);
      b[m] = v < FLT_MIN ? FLT_MIN : v;
    }
    r.fexp[s * r.N * r.E + e] = (short)x;
  }
}

int launch_ripple_f(const RunView &r, const double *tmpl, cudaStream_t st, uint64_t *launches) {
  const size_t cells = (size_t)r.S * r.E * r.M;
  if (r.precision == EPREM_FP64) {
    k_ripple_f<double><<<grid_for(cells), 256, 0, st>>>(r, tmpl);
  } else {
    k_ripple_f<float><<<grid_for(cells), 256, 0, st>>>(r, tmpl);
    k_ripple_rows<<<grid_for((size_t)r.S * r.E), 256, 0, st>>>(r, tmpl);
    *launches += 1;
  }
  *launches += 1;
  return cudaGetLastError() == cudaSuccess ? 0 : EPREM_GPU_ERR_CUDA;
}

// Synthetic seed population: f = sepSeedFunction(E, r) (1 + perturb U) per
// (stream, node, energy), isotropic in mu, with U in (-1, 1) from the top 53
// bits of splitmix64(seed) at index (stream * N + node) * E + energy + 1 --
// the same draw as the workload generator on the host.  Needs seed_radial
// (geometry) of the current positions.
__global__ void k_seed_population(RunView r, unsigned long long seed, double perturb) {
  const size_t SNE = (size_t)r.S * r.N * r.E;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < SNE;
       i += (size_t)gridDim.x * blockDim.x) {
    const size_t g = i / r.E;
    const int e = (int)(i - g * r.E);
    unsigned long long z = seed + (unsigned long long)(i + 1) * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z = z ^ (z >> 31);
    const double u = 2.0 * ((double)(z >> 11) * (1.0 / 9007199254740992.0)) - 1.0;
    const double v = seed_value(r, r.ec[e], r.seed_radial[g]) * (1.0 + perturb * u);
    if (r.precision == EPREM_FP64) {
      double *row = reinterpret_cast<double *>(r.f) + i * r.M;
      for (int m = 0; m < r.M; m++) row[m] = v;
    } else {
      float *row = reinterpret_cast<float *>(r.f) + i * r.M;
      const int x = row_exp_for(ilogb(v));
      const float vf = to_real<float>(ldexp(v, x));
      for (int m = 0; m < r.M; m++) row[m] = vf;
      r.fexp[i] = (short)x;
    }
  }
}

int launch_seed_population(const RunView &r, unsigned long long seed, double perturb,
                           cudaStream_t st, uint64_t *launches) {
  k_seed_population<<<grid_for((size_t)r.S * r.N * r.E), 256, 0, st>>>(r, seed, perturb);
  *launches += 1;
  return cudaGetLastError() == cudaSuccess ? 0 : EPREM_GPU_ERR_CUDA;
}

}  // namespace eprem
