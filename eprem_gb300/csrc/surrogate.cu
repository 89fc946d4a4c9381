// surrogate.cu -- the split focusing + scattering step and its learned
// surrogate (no counterpart in the reference).
//
// Surrogate of the focusing step.  With the relaxation left inside the
// streaming sub-cycles (the reference's scheme), the node-phase row step is
// the focusing alone: the surrogate then changes nothing in the operator
// splitting.
//
// Split form.  The reference relaxes f towards its mu-average inside every
// streaming sub-cycle (src/energeticParticles.c:2406-2426).  In the split
// form streaming runs without it, and the node phase applies, per (node, E)
// row, the focusing sub-cycles (the Euler upwind of k_focus32) followed by
// one exact relaxation over the whole sub-step, f = iso + (f - iso) e with
// e = exp(-dt / tau).  Both pieces conserve sum_mu f.
//
// Surrogate.  A 3-layer MLP (48 -> 256 -> 256 -> 48, tanh-form GELU, bf16
// weights, fp32 accumulation on the tensor cores: mlp.cu) maps the row's
// features -- ln f(mu) minus its mean (40 values), asinh(a dt/dmu),
// asinh(b dt/dmu), 1 - e -- to the change of ln f(mu) over the split step.
// Its output is projected to conserve sum_mu f exactly (FP64 sums), and a
// per-row residual decides whether to keep it: the Crank-Nicolson residual
//   r = f_out - f_in - (dtL(f_in) + dtL(f_out)) / 2,
// L the upwind focusing plus relaxation operator, relative to max f_in; rows
// above the tolerance (calibrated on rows the plain step produced) are
// recomputed by the plain kernel.
#include <cuda_bf16.h>

#include "common.cuh"
#include "kernels.h"

namespace eprem {

constexpr int kSurM = 40;
constexpr int kSurIn = 48;
constexpr int kSurOut = 48;
constexpr int kRowThreads = 128;
// ln f features and ln f changes are clamped: beyond these the row sits at the
// floor, the network's output is not trusted and the residual check sends the
// row to the plain kernel
constexpr float kFeatClamp = 16.f;
constexpr float kTargetClamp = 8.f;

__device__ __forceinline__ float gelu_f(float z) {
  const float u = 0.7978845608f * (z + 0.044715f * z * z * z);
  return 0.5f * z * (1.f + tanhf(u));
}

__device__ __forceinline__ float gelu_grad(float z) {
  const float u = 0.7978845608f * (z + 0.044715f * z * z * z);
  const float t = tanhf(u);
  return 0.5f * (1.f + t) + 0.5f * z * (1.f - t * t) * 0.7978845608f * (1.f + 0.134145f * z * z);
}

// The row's operator: focusing strength a, b (per unit mu velocity,
// src/energeticParticles.c:1620-1627), sub-cycle count and scale, and the
// relaxation factor exp(-dt/tau) with tau = lambda / v.
struct RowOp {
  float a, b, sc, e;
  int ns;
};

__device__ __forceinline__ RowOp row_op(const RunView &r, const NodeCoef32 &c, size_t g, int e) {
  RowOp op;
  const float v = r.ec[e].v32, vi = r.ec[e].vi32;
  op.a = -(v * c.dlnbds) - (2.f * vi) * c.dupar;
  op.b = c.b;
  op.sc = c.scale_f;
  op.ns = c.ns_f;
  // relaxation in the node phase only in the split form; in the reference
  // scheme it stays inside the streaming sub-cycles and the row step is the
  // focusing alone (e = 1)
  const float tau = vi * ((float)r.ec[e].rig_lamo * (float)r.mfp_node[g]);
  op.e = r.relax_in_stream ? 1.f : expf(-(float)r.dt / tau);
  return op;
}

// Plain split step on a 40-cell row in registers.
__device__ __forceinline__ void focus_relax_row(float (&fr)[kSurM], const RowOp &op,
                                                const float *mu32) {
  if (op.ns > 0) {
    float qp[kSurM], qn[kSurM];
    float vel_prev = 0.f;
#pragma unroll
    for (int m = 0; m < kSurM; ++m) {
      const float mu = mu32[m];
      const float vel = 0.5f * (1.f - mu * mu) * (op.a + mu * op.b);
      qp[m] = qn[m] = 0.f;
      if (m >= 1) {
        const float q = op.sc * 0.5f * (vel + vel_prev);
        qp[m] = fmaxf(q, 0.f);
        qn[m] = fminf(q, 0.f);
      }
      vel_prev = vel;
    }
    for (int s = 0; s < op.ns; ++s) {
      float gprev = 0.f;
#pragma unroll
      for (int m = 0; m < kSurM; ++m) {
        float gnext = 0.f;
        if (m + 1 < kSurM) gnext = fmaf(qn[m + 1], fr[m + 1], qp[m + 1] * fr[m]);
        fr[m] = fr[m] - (gnext - gprev);
        gprev = gnext;
      }
    }
  }
  float acc = 0.f;
#pragma unroll
  for (int m = 0; m < kSurM; ++m) acc += fr[m];
  const float iso = (acc * (1.f / kSurM)) * (1.f - op.e);
#pragma unroll
  for (int m = 0; m < kSurM; ++m) fr[m] = fr[m] * op.e + iso;
}

// Features of a row: ln f - mean(ln f), asinh(a dt/dmu), asinh(b dt/dmu), 1-e.
__device__ __forceinline__ void row_features(const float (&lnf)[kSurM], const RowOp &op,
                                             float (&x)[kSurIn]) {
  float mean = 0.f;
#pragma unroll
  for (int m = 0; m < kSurM; ++m) mean += lnf[m];
  mean *= 1.f / kSurM;
#pragma unroll
  for (int m = 0; m < kSurM; ++m) x[m] = fminf(fmaxf(lnf[m] - mean, -kFeatClamp), kFeatClamp);
  const float full = op.sc * (float)op.ns;  // dt / dmu
  x[40] = asinhf(op.a * full);
  x[41] = asinhf(op.b * full);
  x[42] = 1.f - op.e;
#pragma unroll
  for (int m = 43; m < kSurIn; ++m) x[m] = 0.f;
}

// dt L(f)[m] of the split operator for the whole step: upwind focusing with
// face Courant numbers A, B (velocity times dt/dmu) and relaxation at rate
// kappa = dt / tau.
__device__ __forceinline__ float cn_residual(const float (&fin)[kSurM], const float (&fout)[kSurM],
                                             float A, float B, float kappa, const float *mu32) {
  float si = 0.f, so = 0.f, mx = 0.f;
#pragma unroll
  for (int m = 0; m < kSurM; ++m) {
    si += fin[m];
    so += fout[m];
    mx = fmaxf(mx, fin[m]);
  }
  const float isoi = si * (1.f / kSurM), isoo = so * (1.f / kSurM);
  float gi_prev = 0.f, go_prev = 0.f, res = 0.f;
#pragma unroll
  for (int m = 0; m < kSurM; ++m) {
    const float mu = mu32[m];
    const float vel = 0.5f * (1.f - mu * mu) * (A + mu * B);
    float gi = 0.f, go = 0.f;
    if (m + 1 < kSurM) {
      const float mun = mu32[m + 1];
      const float veln = 0.5f * (1.f - mun * mun) * (A + mun * B);
      const float q = 0.5f * (vel + veln);
      gi = q >= 0.f ? q * fin[m] : q * fin[m + 1];
      go = q >= 0.f ? q * fout[m] : q * fout[m + 1];
    }
    const float li = -(gi - gi_prev) - kappa * (fin[m] - isoi);
    const float lo = -(go - go_prev) - kappa * (fout[m] - isoo);
    const float rm = fout[m] - fin[m] - 0.5f * (li + lo);
    res = fmaxf(res, fabsf(rm));
    gi_prev = gi;
    go_prev = go;
  }
  return mx > 0.f ? res / mx : INFINITY;
}

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// ---- plain split step (and the fallback for rejected rows) ------------------
__global__ void __launch_bounds__(kRowThreads)
    k_split_focus_relax(RunView r, size_t row0, size_t nrows, const uint8_t *mask) {
  const size_t i = (size_t)blockIdx.x * kRowThreads + threadIdx.x;
  if (i >= nrows) return;
  if (mask && !mask[i]) return;
  const size_t it = row0 + i;
  const size_t g = it / r.E;
  const int e = (int)(it - g * r.E);
  const NodeCoef32 c = r.coef32[g];
  if (!c.ok) return;
  float *row = reinterpret_cast<float *>(r.f) + it * kSurM;
  float fr[kSurM];
#pragma unroll
  for (int m = 0; m < kSurM; ++m) fr[m] = row[m];
  focus_relax_row(fr, row_op(r, c, g, e), r.mugrid32);
  int code = 0;
#pragma unroll
  for (int m = 0; m < kSurM; ++m) {
    const float v = fr[m];
    if (bad_value(v, &code)) set_error(r, code, 2, (int)(g / r.N), (int)(g % r.N), e, m);
    row[m] = v < FLT_MIN ? FLT_MIN : v;
  }
}

// ---- training samples from the current state --------------------------------
__global__ void __launch_bounds__(kRowThreads)
    k_surr_sample(RunView r, float *xs, float *ts, unsigned long long *count,
                  unsigned long long cap, unsigned long long seed, float rate) {
  const size_t rows = (size_t)r.S * r.N * r.E;
  const size_t it = (size_t)blockIdx.x * kRowThreads + threadIdx.x;
  if (it >= rows) return;
  const double u = (double)(mix64(seed + (it + 1) * 0x9E3779B97F4A7C15ull) >> 11) *
                   (1.0 / 9007199254740992.0);
  if (u >= (double)rate) return;
  const size_t g = it / r.E;
  const int e = (int)(it - g * r.E);
  const NodeCoef32 c = r.coef32[g];
  if (!c.ok || c.ns_f <= 0) return;
  const unsigned long long slot = atomicAdd(count, 1ull);
  if (slot >= cap) return;
  const float *row = reinterpret_cast<const float *>(r.f) + it * kSurM;
  float fr[kSurM], lnf[kSurM], x[kSurIn];
#pragma unroll
  for (int m = 0; m < kSurM; ++m) {
    fr[m] = row[m];
    lnf[m] = logf(fr[m]);
  }
  const RowOp op = row_op(r, c, g, e);
  row_features(lnf, op, x);
  focus_relax_row(fr, op, r.mugrid32);
  float *xo = xs + slot * kSurIn;
  float *to = ts + slot * kSurM;
#pragma unroll
  for (int m = 0; m < kSurIn; ++m) xo[m] = x[m];
#pragma unroll
  for (int m = 0; m < kSurM; ++m)
    to[m] = fminf(fmaxf(logf(fmaxf(fr[m], FLT_MIN)) - lnf[m], -kTargetClamp), kTargetClamp);
}

// ---- inference: features of a chunk of rows ---------------------------------
__global__ void __launch_bounds__(kRowThreads)
    k_surr_features(RunView r, size_t row0, size_t nrows, __nv_bfloat16 *X) {
  const size_t i = (size_t)blockIdx.x * kRowThreads + threadIdx.x;
  if (i >= nrows) return;
  const size_t it = row0 + i;
  const size_t g = it / r.E;
  const int e = (int)(it - g * r.E);
  const NodeCoef32 c = r.coef32[g];
  __nv_bfloat16 *xo = X + i * kSurIn;
  if (!c.ok) {
#pragma unroll
    for (int m = 0; m < kSurIn; ++m) xo[m] = __float2bfloat16_rn(0.f);
    return;
  }
  const float *row = reinterpret_cast<const float *>(r.f) + it * kSurM;
  float lnf[kSurM], x[kSurIn];
#pragma unroll
  for (int m = 0; m < kSurM; ++m) lnf[m] = logf(row[m]);
  row_features(lnf, row_op(r, c, g, e), x);
#pragma unroll
  for (int m = 0; m < kSurIn; ++m) xo[m] = __float2bfloat16_rn(x[m]);
}

// ---- inference: apply the network's output ----------------------------------
// f_out = exp(ln f + y) scaled so that sum_mu f_out = sum_mu f_in (FP64 sums);
// rows whose residual exceeds tol (or are not finite) are left for the plain
// kernel: reject[i] = 1.  counts[0] += kept rows, counts[1] += rejected rows.
__global__ void __launch_bounds__(kRowThreads)
    k_surr_apply(RunView r, size_t row0, size_t nrows, const float *Y, int ldy, float tol,
                 uint8_t *reject, unsigned long long *counts) {
  const size_t i = (size_t)blockIdx.x * kRowThreads + threadIdx.x;
  bool kept = false, rej = false;
  if (i < nrows) {
    const size_t it = row0 + i;
    const size_t g = it / r.E;
    const int e = (int)(it - g * r.E);
    const NodeCoef32 c = r.coef32[g];
    reject[i] = 0;
    if (c.ok) {
      float *row = reinterpret_cast<float *>(r.f) + it * kSurM;
      float fin[kSurM], fout[kSurM];
      double sin_ = 0.0, sout = 0.0;
      const float *y = Y + i * ldy;
#pragma unroll
      for (int m = 0; m < kSurM; ++m) {
        fin[m] = row[m];
        fout[m] = expf(logf(fin[m]) + y[m]);
        sin_ += (double)fin[m];
        sout += (double)fout[m];
      }
      const float scale = (float)(sin_ / sout);
#pragma unroll
      for (int m = 0; m < kSurM; ++m) fout[m] *= scale;
      const RowOp op = row_op(r, c, g, e);
      const float full = op.sc * (float)op.ns;
      const float res = cn_residual(fin, fout, op.a * full, op.b * full, -logf(op.e), r.mugrid32);
      if (res <= tol) {  // false for NaN
        kept = true;
#pragma unroll
        for (int m = 0; m < kSurM; ++m) row[m] = fout[m] < FLT_MIN ? FLT_MIN : fout[m];
      } else {
        rej = true;
        reject[i] = 1;
      }
    }
  }
  const unsigned full_mask = 0xffffffffu;
  const unsigned k = __popc(__ballot_sync(full_mask, kept));
  const unsigned j = __popc(__ballot_sync(full_mask, rej));
  if ((threadIdx.x & 31) == 0) {
    if (k) atomicAdd(&counts[0], (unsigned long long)k);
    if (j) atomicAdd(&counts[1], (unsigned long long)j);
  }
}

// Residual of (features, target change) pairs: the tolerance calibration on
// rows the plain step produced.
__global__ void k_surr_residual(const float *xs, const float *ts, size_t n, const float *mu32,
                                float *res) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float *x = xs + i * kSurIn;
  const float *t = ts + i * kSurM;
  float fin[kSurM], fout[kSurM];
#pragma unroll
  for (int m = 0; m < kSurM; ++m) {
    fin[m] = expf(x[m]);
    fout[m] = expf(x[m] + t[m]);
  }
  const float e = 1.f - x[42];
  res[i] = cn_residual(fin, fout, sinhf(x[40]), sinhf(x[41]), -logf(e), mu32);
}

// ---- network elementwise kernels ---------------------------------------------
__global__ void k_to_bf16(const float *in, __nv_bfloat16 *out, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    out[i] = __float2bfloat16_rn(in[i]);
}

__global__ void k_gelu_bf16(const float *Z, __nv_bfloat16 *H, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    H[i] = __float2bfloat16_rn(gelu_f(Z[i]));
}

// dY = 2 (Y - T) / (rows * 40) on the 40 used outputs, 0 on the padding; the
// squared error is summed into *loss.
__global__ void k_mse_grad(const float *Y, const float *T, size_t rows, float *dY,
                           __nv_bfloat16 *dYb, double *loss) {
  const size_t n = rows * kSurOut;
  double part = 0.0;
  const float scale = 2.f / (float)(rows * kSurM);
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const size_t row = i / kSurOut;
    const int col = (int)(i - row * kSurOut);
    float d = 0.f;
    if (col < kSurM) {
      const float diff = Y[i] - T[row * kSurM + col];
      part += (double)diff * diff;
      d = scale * diff;
    }
    dY[i] = d;
    dYb[i] = __float2bfloat16_rn(d);
  }
  for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
  if ((threadIdx.x & 31) == 0 && part != 0.0) atomicAdd(loss, part);
}

// dZ = dH * gelu'(Z), fp32 and bf16 copies
__global__ void k_gelu_back(const float *dH, const float *Z, float *dZ, __nv_bfloat16 *dZb,
                            size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const float d = dH[i] * gelu_grad(Z[i]);
    dZ[i] = d;
    dZb[i] = __float2bfloat16_rn(d);
  }
}

// out[c][r] = in[r][c] for an R x C bf16 matrix (32 x 32 tiles)
__global__ void k_transpose_bf16(const __nv_bfloat16 *in, __nv_bfloat16 *out, int R, int C) {
  __shared__ __nv_bfloat16 tile[32][33];
  const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int rr = r0 + j, cc = c0 + threadIdx.x;
    if (rr < R && cc < C) tile[j][threadIdx.x] = in[(size_t)rr * C + cc];
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int cc = c0 + j, rr = r0 + threadIdx.x;
    if (rr < R && cc < C) out[(size_t)cc * R + rr] = tile[threadIdx.x][j];
  }
}

// out[c] = sum_r in[r][c] for an R x C fp32 matrix (one thread per column,
// FP64 accumulation)
__global__ void k_colsum(const float *in, int R, int C, float *out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= C) return;
  double s = 0.0;
  for (int r = 0; r < R; r++) s += (double)in[(size_t)r * C + c];
  out[c] = (float)s;
}

__global__ void k_adam(float *p, const float *g, float *m, float *v, size_t n, float lr, float b1,
                       float b2, float eps, float c1, float c2) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

// ---- host-side launchers -----------------------------------------------------
static unsigned blocks_for(size_t n, int threads) {
  size_t b = (n + threads - 1) / threads;
  return (unsigned)(b > (1u << 20) ? (1u << 20) : (b ? b : 1));
}

int launch_split_focus_relax(const RunView &r, size_t row0, size_t nrows, const uint8_t *mask,
                             cudaStream_t st, uint64_t *launches) {
  k_split_focus_relax<<<(unsigned)((nrows + kRowThreads - 1) / kRowThreads), kRowThreads, 0, st>>>(
      r, row0, nrows, mask);
  *launches += 1;
  return cudaGetLastError() == cudaSuccess ? 0 : EPREM_GPU_ERR_CUDA;
}

int launch_surr_sample(const RunView &r, float *xs, float *ts, unsigned long long *count,
                       unsigned long long cap, unsigned long long seed, float rate,
                       cudaStream_t st) {
  const size_t rows = (size_t)r.S * r.N * r.E;
  k_surr_sample<<<(unsigned)((rows + kRowThreads - 1) / kRowThreads), kRowThreads, 0, st>>>(
      r, xs, ts, count, cap, seed, rate);
  return cudaGetLastError() == cudaSuccess ? 0 : EPREM_GPU_ERR_CUDA;
}

int launch_surr_features(const RunView &r, size_t row0, size_t nrows, void *X, cudaStream_t st,
                         uint64_t *launches) {
  k_surr_features<<<(unsigned)((nrows + kRowThreads - 1) / kRowThreads), kRowThreads, 0, st>>>(
      r, row0, nrows, static_cast<__nv_bfloat16 *>(X));
  *launches += 1;
  return cudaGetLastError() == cudaSuccess ? 0 : EPREM_GPU_ERR_CUDA;
}

int launch_surr_apply(const RunView &r, size_t row0, size_t nrows, const float *Y, int ldy,
                      float tol, uint8_t *reject, unsigned long long *counts, cudaStream_t st,
                      uint64_t *launches) {
  k_surr_apply<<<(unsigned)((nrows + kRowThreads - 1) / kRowThreads), kRowThreads, 0, st>>>(
      r, row0, nrows, Y, ldy, tol, reject, counts);
  *launches += 1;
  return cudaGetLastError() == cudaSuccess ? 0 : EPREM_GPU_ERR_CUDA;
}

// The acceptance check's statistic and the true error of the network's output on
// collected rows, whose plain step (the target) is known: for row i the
// residual of the network's projected output (as k_surr_apply forms it) and
// its distance from the plain step, max over mu of |f_net - f_plain|
// relative to the plain row's mean.
__global__ void k_surr_calib(const float *xs, const float *ts, const float *Y, int ldy,
                             size_t n, const float *mu32, float *res, float *err) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float *x = xs + i * kSurIn;
  const float *t = ts + i * kSurM;
  const float *y = Y + i * ldy;
  float fin[kSurM], fout[kSurM];
  double sin_ = 0.0, sout = 0.0, splain = 0.0;
#pragma unroll
  for (int m = 0; m < kSurM; ++m) {
    fin[m] = expf(x[m]);
    fout[m] = expf(x[m] + y[m]);
    sin_ += (double)fin[m];
    sout += (double)fout[m];
    splain += (double)expf(x[m] + t[m]);
  }
  const float scale = (float)(sin_ / sout);
  float dmax = 0.f;
#pragma unroll
  for (int m = 0; m < kSurM; ++m) {
    fout[m] *= scale;
    dmax = fmaxf(dmax, fabsf(fout[m] - expf(x[m] + t[m])));
  }
  const float e = 1.f - x[42];
  res[i] = cn_residual(fin, fout, sinhf(x[40]), sinhf(x[41]), -logf(e), mu32);
  err[i] = (float)(dmax / (splain / kSurM));
}

int launch_surr_calib(const float *xs, const float *ts, const float *Y, int ldy, size_t n,
                      const float *mu32, float *res, float *err, cudaStream_t st) {
  k_surr_calib<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(xs, ts, Y, ldy, n, mu32, res, err);
  return cudaGetLastError() == cudaSuccess ? 0 : EPREM_GPU_ERR_CUDA;
}

int launch_surr_residual(const float *xs, const float *ts, size_t n, const float *mu32,
                         float *res, cudaStream_t st) {
  k_surr_residual<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(xs, ts, n, mu32, res);
  return cudaGetLastError() == cudaSuccess ? 0 : EPREM_GPU_ERR_CUDA;
}

int launch_to_bf16(const float *in, void *out, size_t n, cudaStream_t st) {
  k_to_bf16<<<blocks_for(n, 256), 256, 0, st>>>(in, static_cast<__nv_bfloat16 *>(out), n);
  return cudaGetLastError() == cudaSuccess ? 0 : EPREM_GPU_ERR_CUDA;
}

int launch_gelu_bf16(const float *Z, void *H, size_t n, cudaStream_t st) {
  k_gelu_bf16<<<blocks_for(n, 256), 256, 0, st>>>(Z, static_cast<__nv_bfloat16 *>(H), n);
  return cudaGetLastError() == cudaSuccess ? 0 : EPREM_GPU_ERR_CUDA;
}

int launch_mse_grad(const float *Y, const float *T, size_t rows, float *dY, void *dYb,
                    double *loss, cudaStream_t st) {
  k_mse_grad<<<blocks_for(rows * kSurOut, 256), 256, 0, st>>>(
      Y, T, rows, dY, static_cast<__nv_bfloat16 *>(dYb), loss);
  return cudaGetLastError() == cudaSuccess ? 0 : EPREM_GPU_ERR_CUDA;
}

int launch_gelu_back(const float *dH, const float *Z, float *dZ, void *dZb, size_t n,
                     cudaStream_t st) {
  k_gelu_back<<<blocks_for(n, 256), 256, 0, st>>>(dH, Z, dZ, static_cast<__nv_bfloat16 *>(dZb), n);
  return cudaGetLastError() == cudaSuccess ? 0 : EPREM_GPU_ERR_CUDA;
}

int launch_transpose_bf16(const void *in, void *out, int R, int C, cudaStream_t st) {
  dim3 grid((C + 31) / 32, (R + 31) / 32);
  k_transpose_bf16<<<grid, dim3(32, 8), 0, st>>>(static_cast<const __nv_bfloat16 *>(in),
                                                 static_cast<__nv_bfloat16 *>(out), R, C);
  return cudaGetLastError() == cudaSuccess ? 0 : EPREM_GPU_ERR_CUDA;
}

int launch_colsum(const float *in, int R, int C, float *out, cudaStream_t st) {
  k_colsum<<<(C + 127) / 128, 128, 0, st>>>(in, R, C, out);
  return cudaGetLastError() == cudaSuccess ? 0 : EPREM_GPU_ERR_CUDA;
}

int launch_adam(float *p, const float *g, float *m, float *v, size_t n, float lr, int step,
                cudaStream_t st) {
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
  k_adam<<<blocks_for(n, 256), 256, 0, st>>>(p, g, m, v, n, lr, b1, b2, 1e-8f, c1, c2);
  return cudaGetLastError() == cudaSuccess ? 0 : EPREM_GPU_ERR_CUDA;
}

}  // namespace eprem
