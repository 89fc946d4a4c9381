// surrogate_host.cu -- the ABI of the split form and the learned surrogate:
// the network's parameters and training loop, the training set, the node
// phase of the split and surrogate forms (kernels in surrogate.cu, mlp.cu).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "run.h"

using namespace eprem;

// ---- surrogate building blocks ---------------------------------------------
namespace {
std::mutex g_gemm_err_mutex;
int *g_gemm_err[kMaxDevices] = {};
}  // namespace

extern "C" int eprem_gpu_gemm_bf16(const void *A, int lda, const void *Bt, int ldb,
                                   const float *bias, float *C, int ldc, int M, int N, int K,
                                   void *stream) {
  if (!A || !Bt || !C) return fail(EPREM_GPU_ERR_ARG, "null operand");
  int dev = 0;
  CK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return fail(EPREM_GPU_ERR_ARG, "device ordinal");
  int *err = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_gemm_err_mutex);
    if (!g_gemm_err[dev]) CK(cudaMalloc(&g_gemm_err[dev], sizeof(int)));
    err = g_gemm_err[dev];
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  CK(cudaMemsetAsync(err, 0, sizeof(int), st));
  const int rc = launch_gemm_bf16(A, lda, Bt, ldb, bias, C, ldc, M, N, K, err, st);
  if (rc == EPREM_GPU_ERR_ARG)
    return fail(rc, "gemm shape: K, lda, ldb multiples of 8, lda/ldb >= K, ldc >= N");
  if (rc) return cuda_fail(cudaGetLastError(), "gemm launch");
  int h = 0;
  CK(cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (h) return fail(EPREM_GPU_ERR_CUDA, "gemm: wait on the tensor cores timed out");
  return EPREM_GPU_OK;
}


// ---- learned surrogate -------------------------------------------------------
// Network 48 -> 256 -> 256 -> 48; parameters flat in fp32:
// W1t[256][48], b1[256], W2t[256][256], b2[256], W3t[48][256], b3[48]
// (Wt[out][in]).  bf16 copies: Wt for the forward GEMMs (Bt operands of
// shape out x in), W2 and W3 (in x out) for the backward data gradients.
namespace {
constexpr int kSIn = 48, kSHid = 256, kSOut = 48, kSM = 40;
constexpr size_t kOffW1 = 0, kOffB1 = kOffW1 + (size_t)kSHid * kSIn, kOffW2 = kOffB1 + kSHid,
                 kOffB2 = kOffW2 + (size_t)kSHid * kSHid, kOffW3 = kOffB2 + kSHid,
                 kOffB3 = kOffW3 + (size_t)kSOut * kSHid, kNParams = kOffB3 + kSOut;
constexpr int kBatchMax = 16384;
typedef uint16_t bf16_t;

uint64_t splitmix(uint64_t &state) {
  uint64_t z = (state += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
}  // namespace

struct eprem_gpu_surrogate {
  int device = 0;
  cudaStream_t st = nullptr;
  float *p = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;
  bf16_t *w1t = nullptr, *w2t = nullptr, *w3t = nullptr, *w2 = nullptr, *w3 = nullptr;
  // training samples
  float *xs = nullptr, *ts = nullptr;
  unsigned long long *d_count = nullptr;
  size_t cap = 0, n = 0;
  // inference chunk buffers (R rows)
  size_t R = 0;
  bf16_t *X = nullptr, *Ha = nullptr, *Hb = nullptr;
  float *Z = nullptr, *Y = nullptr;
  // training batch buffers (kBatchMax rows)
  bf16_t *tX, *tXt, *tH1, *tH1t, *tH2, *tH2t, *tdYb, *tdYt, *tdZb, *tdZt;
  float *tZ1, *tZ2, *tY, *tdY, *tdH, *tdZ, *tT;
  double *d_loss = nullptr;
  int *d_err = nullptr;
  DevStatus *scratch_status = nullptr;
  float *mu32 = nullptr;  // the uniform 40-cell mu grid
  float tol = 0.f;
  int step = 0;
  uint64_t rng = 0;
  std::vector<void *> allocs;
};

template <typename T>
static cudaError_t salloc(eprem_gpu_surrogate *s, T **ptr, size_t n) {
  cudaError_t e = cudaMalloc(reinterpret_cast<void **>(ptr), n * sizeof(T) + 16);
  if (e == cudaSuccess) s->allocs.push_back(*ptr);
  return e;
}

extern "C" int64_t eprem_gpu_surrogate_num_params(void) { return (int64_t)kNParams; }

extern "C" int eprem_gpu_surrogate_destroy(eprem_gpu_surrogate *s) {
  if (!s) return EPREM_GPU_OK;
  if (s->st) cudaStreamSynchronize(s->st);
  for (void *ptr : s->allocs) cudaFree(ptr);
  if (s->st) cudaStreamDestroy(s->st);
  delete s;
  return EPREM_GPU_OK;
}

// bf16 forward / backward weight copies from the fp32 master parameters
static int surr_sync_weights(eprem_gpu_surrogate *s) {
  if (launch_to_bf16(s->p + kOffW1, s->w1t, (size_t)kSHid * kSIn, s->st) ||
      launch_to_bf16(s->p + kOffW2, s->w2t, (size_t)kSHid * kSHid, s->st) ||
      launch_to_bf16(s->p + kOffW3, s->w3t, (size_t)kSOut * kSHid, s->st) ||
      launch_transpose_bf16(s->w2t, s->w2, kSHid, kSHid, s->st) ||
      launch_transpose_bf16(s->w3t, s->w3, kSOut, kSHid, s->st))
    return cuda_fail(cudaGetLastError(), "surrogate weight copies");
  return EPREM_GPU_OK;
}

extern "C" int eprem_gpu_surrogate_create(uint64_t seed, int chunk_rows,
                                          eprem_gpu_surrogate **out) {
  if (!out) return fail(EPREM_GPU_ERR_ARG, "null output handle");
  *out = nullptr;
  if (chunk_rows <= 0) chunk_rows = 1 << 19;
  auto *s = new eprem_gpu_surrogate();
  s->R = (size_t)((chunk_rows + 127) / 128) * 128;
  s->rng = seed;
  cudaError_t e = cudaGetDevice(&s->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = salloc(s, &s->p, kNParams);
  if (e == cudaSuccess) e = salloc(s, &s->g, kNParams);
  if (e == cudaSuccess) e = salloc(s, &s->m, kNParams);
  if (e == cudaSuccess) e = salloc(s, &s->v, kNParams);
  if (e == cudaSuccess) e = salloc(s, &s->w1t, (size_t)kSHid * kSIn);
  if (e == cudaSuccess) e = salloc(s, &s->w2t, (size_t)kSHid * kSHid);
  if (e == cudaSuccess) e = salloc(s, &s->w3t, (size_t)kSOut * kSHid);
  if (e == cudaSuccess) e = salloc(s, &s->w2, (size_t)kSHid * kSHid);
  if (e == cudaSuccess) e = salloc(s, &s->w3, (size_t)kSHid * kSOut);
  if (e == cudaSuccess) e = salloc(s, &s->X, s->R * kSIn);
  if (e == cudaSuccess) e = salloc(s, &s->Ha, s->R * kSHid);
  if (e == cudaSuccess) e = salloc(s, &s->Hb, s->R * kSHid);
  if (e == cudaSuccess) e = salloc(s, &s->Z, s->R * kSHid);
  if (e == cudaSuccess) e = salloc(s, &s->Y, s->R * kSOut);
  const size_t B = kBatchMax;
  bf16_t **bb[] = {&s->tX, &s->tXt, &s->tH1, &s->tH1t, &s->tH2, &s->tH2t, &s->tdYb, &s->tdYt,
                   &s->tdZb, &s->tdZt};
  const size_t bn[] = {B * kSIn, B * kSIn, B * kSHid, B * kSHid, B * kSHid, B * kSHid,
                       B * kSOut, B * kSOut, B * kSHid, B * kSHid};
  for (int i = 0; i < 10 && e == cudaSuccess; i++) e = salloc(s, bb[i], bn[i]);
  float **ff[] = {&s->tZ1, &s->tZ2, &s->tY, &s->tdY, &s->tdH, &s->tdZ, &s->tT};
  const size_t fn[] = {B * kSHid, B * kSHid, B * kSOut, B * kSOut, B * kSHid, B * kSHid, B * kSM};
  for (int i = 0; i < 7 && e == cudaSuccess; i++) e = salloc(s, ff[i], fn[i]);
  if (e == cudaSuccess) e = salloc(s, &s->d_loss, 1);
  if (e == cudaSuccess) e = salloc(s, &s->d_err, 1);
  if (e == cudaSuccess) e = salloc(s, &s->d_count, 1);
  if (e == cudaSuccess) e = salloc(s, &s->scratch_status, 1);
  if (e == cudaSuccess) e = salloc(s, &s->mu32, kSM);
  // Xavier-uniform weights from splitmix64(seed), zero biases; the output
  // layer starts at a tenth of that so the initial change of ln f is small
  std::vector<float> h(kNParams, 0.f);
  auto fill = [&](size_t off, int fan_out, int fan_in, float gain) {
    const double a = gain * std::sqrt(6.0 / (fan_in + fan_out));
    for (size_t i = 0; i < (size_t)fan_out * fan_in; i++) {
      const double u = (double)(splitmix(s->rng) >> 11) * (1.0 / 9007199254740992.0);
      h[off + i] = (float)((2.0 * u - 1.0) * a);
    }
  };
  fill(kOffW1, kSHid, kSIn, 1.f);
  fill(kOffW2, kSHid, kSHid, 1.f);
  fill(kOffW3, kSOut, kSHid, 0.1f);
  std::vector<float> mu(kSM);
  for (int i = 0; i < kSM; i++) mu[i] = (float)(-1.0 + (i + 0.5) * (2.0 / kSM));
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(s->p, h.data(), kNParams * sizeof(float), cudaMemcpyHostToDevice, s->st);
  if (e == cudaSuccess) e = cudaMemsetAsync(s->m, 0, kNParams * sizeof(float), s->st);
  if (e == cudaSuccess) e = cudaMemsetAsync(s->v, 0, kNParams * sizeof(float), s->st);
  if (e == cudaSuccess) e = cudaMemsetAsync(s->d_count, 0, sizeof(unsigned long long), s->st);
  if (e == cudaSuccess) e = cudaMemsetAsync(s->d_err, 0, sizeof(int), s->st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(s->mu32, mu.data(), kSM * sizeof(float), cudaMemcpyHostToDevice, s->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->st);
  if (e != cudaSuccess) {
    eprem_gpu_surrogate_destroy(s);
    return cuda_fail(e, "eprem_gpu_surrogate_create");
  }
  int rc = surr_sync_weights(s);
  if (rc == EPREM_GPU_OK && cudaStreamSynchronize(s->st) != cudaSuccess)
    rc = cuda_fail(cudaGetLastError(), "eprem_gpu_surrogate_create");
  if (rc) {
    eprem_gpu_surrogate_destroy(s);
    return rc;
  }
  *out = s;
  return EPREM_GPU_OK;
}

extern "C" int eprem_gpu_surrogate_get_params(eprem_gpu_surrogate *s, float *host, int64_t n) {
  if (!s || !host || n != (int64_t)kNParams) return fail(EPREM_GPU_ERR_ARG, "params: size");
  CK(cudaMemcpyAsync(host, s->p, kNParams * sizeof(float), cudaMemcpyDeviceToHost, s->st));
  CK(cudaStreamSynchronize(s->st));
  return EPREM_GPU_OK;
}

extern "C" int eprem_gpu_surrogate_set_params(eprem_gpu_surrogate *s, const float *host,
                                              int64_t n) {
  if (!s || !host || n != (int64_t)kNParams) return fail(EPREM_GPU_ERR_ARG, "params: size");
  CK(cudaMemcpyAsync(s->p, host, kNParams * sizeof(float), cudaMemcpyHostToDevice, s->st));
  const int rc = surr_sync_weights(s);
  if (rc) return rc;
  CK(cudaStreamSynchronize(s->st));
  return EPREM_GPU_OK;
}

extern "C" int eprem_gpu_surrogate_reserve(eprem_gpu_surrogate *s, int64_t capacity) {
  if (!s || capacity <= 0) return fail(EPREM_GPU_ERR_ARG, "reserve: capacity");
  CK(cudaStreamSynchronize(s->st));
  if ((size_t)capacity != s->cap) {
    for (void *ptr : {(void *)s->xs, (void *)s->ts})
      for (size_t i = 0; i < s->allocs.size(); i++)
        if (s->allocs[i] == ptr) {
          cudaFree(ptr);
          s->allocs.erase(s->allocs.begin() + i);
          break;
        }
    s->xs = s->ts = nullptr;
    s->cap = 0;
    CK(salloc(s, &s->xs, (size_t)capacity * kSIn));
    CK(salloc(s, &s->ts, (size_t)capacity * kSM));
    s->cap = (size_t)capacity;
  }
  s->n = 0;
  CK(cudaMemsetAsync(s->d_count, 0, sizeof(unsigned long long), s->st));
  CK(cudaStreamSynchronize(s->st));
  return EPREM_GPU_OK;
}

static int surr_check_run(const eprem_gpu_run *r) {
  if (!r->nplan.fast32 || r->dims.num_mu != kSM || !r->v.use_focus)
    return fail(EPREM_GPU_ERR_UNSUPPORTED,
                "the surrogate covers the FP32 form with Euler operators, focusing on and "
                "40 mu cells");
  return EPREM_GPU_OK;
}

// Rows of the run's current state and their plain split step, sampled at
// `rate` (hash of seed and row): the training set.
extern "C" int eprem_gpu_surrogate_collect(eprem_gpu_surrogate *s, eprem_gpu_run *r,
                                           double rate, uint64_t seed, int64_t *total) {
  if (!s || !r) return fail(EPREM_GPU_ERR_ARG, "null argument");
  int rc = surr_check_run(r);
  if (rc) return rc;
  if (!s->cap) return fail(EPREM_GPU_ERR_STATE, "eprem_gpu_surrogate_reserve first");
  const eprem_params_t &p = r->params;
  RunView v = r->v;
  v.status = s->scratch_status;  // the run's statistics stay untouched
  uint64_t dummy = 0;
  CK(cudaMemsetAsync(s->scratch_status, 0, sizeof(DevStatus), r->stream));
  if (launch_geometry(v, r->stream, r->norm_radius, r->neg_beta, p.mfp_type,
                      p.mfp_type == 2 ? p.mfp_b_power : p.mfp_radial_power, p.mhd_bs_au, &dummy) ||
      launch_node32_setup(v, r->stream, &dummy) ||
      launch_surr_sample(v, s->xs, s->ts, s->d_count, s->cap, seed, (float)rate, r->stream))
    return cuda_fail(cudaGetLastError(), "surrogate sample launch");
  unsigned long long c = 0;
  CK(cudaMemcpyAsync(&c, s->d_count, sizeof(c), cudaMemcpyDeviceToHost, r->stream));
  CK(cudaStreamSynchronize(r->stream));
  s->n = c < s->cap ? (size_t)c : s->cap;
  if (total) *total = (int64_t)s->n;
  return EPREM_GPU_OK;
}

// Forward pass of `rows` training rows from xs (fp32 features), keeping the
// activations of the backward pass.
static int surr_forward_train(eprem_gpu_surrogate *s, const float *xs, int rows) {
  cudaStream_t st = s->st;
  const size_t B = (size_t)rows;
  if (launch_to_bf16(xs, s->tX, B * kSIn, st) ||
      launch_gemm_bf16(s->tX, kSIn, s->w1t, kSIn, s->p + kOffB1, s->tZ1, kSHid, rows, kSHid, kSIn,
                       s->d_err, st) ||
      launch_gelu_bf16(s->tZ1, s->tH1, B * kSHid, st) ||
      launch_gemm_bf16(s->tH1, kSHid, s->w2t, kSHid, s->p + kOffB2, s->tZ2, kSHid, rows, kSHid,
                       kSHid, s->d_err, st) ||
      launch_gelu_bf16(s->tZ2, s->tH2, B * kSHid, st) ||
      launch_gemm_bf16(s->tH2, kSHid, s->w3t, kSHid, s->p + kOffB3, s->tY, kSOut, rows, kSOut,
                       kSHid, s->d_err, st))
    return EPREM_GPU_ERR_CUDA;
  return EPREM_GPU_OK;
}

// Loss and gradients of `rows` rows (targets T, fp32 [rows][40]) into s->g.
static int surr_backward(eprem_gpu_surrogate *s, const float *T, int rows) {
  cudaStream_t st = s->st;
  const size_t B = (size_t)rows;
  if (cudaMemsetAsync(s->d_loss, 0, sizeof(double), st) != cudaSuccess ||
      launch_mse_grad(s->tY, T, B, s->tdY, s->tdYb, s->d_loss, st) ||
      // output layer
      launch_transpose_bf16(s->tdYb, s->tdYt, rows, kSOut, st) ||
      launch_transpose_bf16(s->tH2, s->tH2t, rows, kSHid, st) ||
      launch_gemm_bf16(s->tdYt, rows, s->tH2t, rows, nullptr, s->g + kOffW3, kSHid, kSOut, kSHid,
                       rows, s->d_err, st) ||
      launch_colsum(s->tdY, rows, kSOut, s->g + kOffB3, st) ||
      launch_gemm_bf16(s->tdYb, kSOut, s->w3, kSOut, nullptr, s->tdH, kSHid, rows, kSHid, kSOut,
                       s->d_err, st) ||
      launch_gelu_back(s->tdH, s->tZ2, s->tdZ, s->tdZb, B * kSHid, st) ||
      // hidden layer 2
      launch_transpose_bf16(s->tdZb, s->tdZt, rows, kSHid, st) ||
      launch_transpose_bf16(s->tH1, s->tH1t, rows, kSHid, st) ||
      launch_gemm_bf16(s->tdZt, rows, s->tH1t, rows, nullptr, s->g + kOffW2, kSHid, kSHid, kSHid,
                       rows, s->d_err, st) ||
      launch_colsum(s->tdZ, rows, kSHid, s->g + kOffB2, st) ||
      launch_gemm_bf16(s->tdZb, kSHid, s->w2, kSHid, nullptr, s->tdH, kSHid, rows, kSHid, kSHid,
                       s->d_err, st) ||
      launch_gelu_back(s->tdH, s->tZ1, s->tdZ, s->tdZb, B * kSHid, st) ||
      // input layer
      launch_transpose_bf16(s->tdZb, s->tdZt, rows, kSHid, st) ||
      launch_transpose_bf16(s->tX, s->tXt, rows, kSIn, st) ||
      launch_gemm_bf16(s->tdZt, rows, s->tXt, rows, nullptr, s->g + kOffW1, kSIn, kSHid, kSIn,
                       rows, s->d_err, st) ||
      launch_colsum(s->tdZ, rows, kSHid, s->g + kOffB1, st))
    return EPREM_GPU_ERR_CUDA;
  return EPREM_GPU_OK;
}

static int surr_read_err(eprem_gpu_surrogate *s) {
  int h = 0;
  CK(cudaMemcpyAsync(&h, s->d_err, sizeof(int), cudaMemcpyDeviceToHost, s->st));
  CK(cudaStreamSynchronize(s->st));
  if (h) {
    cudaMemsetAsync(s->d_err, 0, sizeof(int), s->st);
    return fail(EPREM_GPU_ERR_CUDA, "surrogate GEMM: wait on the tensor cores timed out");
  }
  return EPREM_GPU_OK;
}

extern "C" int eprem_gpu_surrogate_loss_grad(eprem_gpu_surrogate *s, const float *x_host,
                                             const float *t_host, int rows, double *loss,
                                             float *grad_host) {
  if (!s || !x_host || !t_host || rows <= 0 || rows > kBatchMax || rows % 8)
    return fail(EPREM_GPU_ERR_ARG, "loss_grad: rows must be a multiple of 8, <= 16384");
  CK(cudaMemcpyAsync(s->tT, t_host, (size_t)rows * kSM * sizeof(float), cudaMemcpyHostToDevice,
                     s->st));
  float *xd = s->tdH;  // staging for the fp32 features (rows * 48 <= rows * 256)
  CK(cudaMemcpyAsync(xd, x_host, (size_t)rows * kSIn * sizeof(float), cudaMemcpyHostToDevice,
                     s->st));
  CK(cudaMemsetAsync(s->g, 0, kNParams * sizeof(float), s->st));
  if (surr_forward_train(s, xd, rows) || surr_backward(s, s->tT, rows))
    return cuda_fail(cudaGetLastError(), "surrogate forward/backward");
  double l = 0.0;
  CK(cudaMemcpyAsync(&l, s->d_loss, sizeof(double), cudaMemcpyDeviceToHost, s->st));
  if (grad_host)
    CK(cudaMemcpyAsync(grad_host, s->g, kNParams * sizeof(float), cudaMemcpyDeviceToHost, s->st));
  const int rc = surr_read_err(s);
  if (rc) return rc;
  if (loss) *loss = l / ((double)rows * kSM);
  return EPREM_GPU_OK;
}

extern "C" int eprem_gpu_surrogate_evaluate(eprem_gpu_surrogate *s, const float *x_host, int rows,
                                            float *y_host) {
  if (!s || !x_host || !y_host || rows <= 0 || rows > kBatchMax)
    return fail(EPREM_GPU_ERR_ARG, "evaluate: rows <= 16384");
  float *xd = s->tdH;
  CK(cudaMemcpyAsync(xd, x_host, (size_t)rows * kSIn * sizeof(float), cudaMemcpyHostToDevice,
                     s->st));
  if (surr_forward_train(s, xd, rows)) return cuda_fail(cudaGetLastError(), "surrogate forward");
  CK(cudaMemcpyAsync(y_host, s->tY, (size_t)rows * kSOut * sizeof(float), cudaMemcpyDeviceToHost,
                     s->st));
  return surr_read_err(s);
}

// `steps` Adam steps on random windows of `batch` collected samples.
extern "C" int eprem_gpu_surrogate_train(eprem_gpu_surrogate *s, int steps, int batch, double lr,
                                         double *last_loss) {
  if (!s || steps <= 0 || batch <= 0 || batch > kBatchMax || batch % 8)
    return fail(EPREM_GPU_ERR_ARG, "train: batch a multiple of 8, <= 16384");
  if (s->n < (size_t)batch) return fail(EPREM_GPU_ERR_STATE, "train: fewer samples than a batch");
  double l = 0.0;
  for (int it = 0; it < steps; it++) {
    const size_t off = (size_t)(splitmix(s->rng) % (uint64_t)(s->n - batch + 1));
    if (surr_forward_train(s, s->xs + off * kSIn, batch) ||
        surr_backward(s, s->ts + off * kSM, batch) ||
        launch_adam(s->p, s->g, s->m, s->v, kNParams, (float)lr, ++s->step, s->st))
      return cuda_fail(cudaGetLastError(), "surrogate training step");
    const int rc = surr_sync_weights(s);
    if (rc) return rc;
    if (it == steps - 1) {
      CK(cudaMemcpyAsync(&l, s->d_loss, sizeof(double), cudaMemcpyDeviceToHost, s->st));
    }
  }
  const int rc = surr_read_err(s);
  if (rc) return rc;
  if (last_loss) *last_loss = l / ((double)batch * kSM);
  return EPREM_GPU_OK;
}

// Tolerance of the residual check: the `quantile` of the residuals of the
// collected plain-step rows, times `margin`.
extern "C" int eprem_gpu_surrogate_calibrate(eprem_gpu_surrogate *s, double quantile,
                                             double margin, double *tol_out) {
  if (!s || !s->n) return fail(EPREM_GPU_ERR_STATE, "calibrate: no samples");
  float *res = nullptr;
  CK(cudaMalloc(&res, s->n * sizeof(float)));
  std::vector<float> h(s->n);
  int rc = launch_surr_residual(s->xs, s->ts, s->n, s->mu32, res, s->st);
  cudaError_t e = rc ? cudaGetLastError()
                     : cudaMemcpyAsync(h.data(), res, s->n * sizeof(float),
                                       cudaMemcpyDeviceToHost, s->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->st);
  cudaFree(res);
  if (e != cudaSuccess) return cuda_fail(e, "calibrate");
  std::sort(h.begin(), h.end());
  const size_t k = std::min(h.size() - 1, (size_t)(quantile * (double)(h.size() - 1)));
  s->tol = (float)(h[k] * margin);
  if (tol_out) *tol_out = s->tol;
  return EPREM_GPU_OK;
}

// Tolerance of the residual check from the rows' true error: the network
// runs on up to `rows` collected rows (whose plain step is known), and the
// tolerance is the largest residual below which every row is within
// `target` of its plain step (max over mu, relative to the row's mean).
// *kept: the fraction of those rows the check then keeps; *within: the
// fraction within target at all (what an exact check would keep).
extern "C" int eprem_gpu_surrogate_calibrate_error(eprem_gpu_surrogate *s, double target,
                                                   int64_t rows, double *tol_out,
                                                   double *kept, double *within) {
  if (!s || !s->n) return fail(EPREM_GPU_ERR_STATE, "calibrate: no samples");
  const size_t n = std::min(s->n, rows > 0 ? (size_t)rows : s->n);
  float *res = nullptr, *err = nullptr;
  CK(cudaMalloc(&res, n * sizeof(float)));
  cudaError_t e = cudaMalloc(&err, n * sizeof(float));
  for (size_t r0 = 0; r0 < n && e == cudaSuccess; r0 += s->R) {
    const size_t nr = std::min(s->R, n - r0);
    const int nn = (int)nr;
    if (launch_to_bf16(s->xs + r0 * kSIn, s->X, nr * kSIn, s->st) ||
        launch_gemm_bf16(s->X, kSIn, s->w1t, kSIn, s->p + kOffB1, s->Z, kSHid, nn, kSHid, kSIn,
                         s->d_err, s->st) ||
        launch_gelu_bf16(s->Z, s->Ha, nr * kSHid, s->st) ||
        launch_gemm_bf16(s->Ha, kSHid, s->w2t, kSHid, s->p + kOffB2, s->Z, kSHid, nn, kSHid,
                         kSHid, s->d_err, s->st) ||
        launch_gelu_bf16(s->Z, s->Hb, nr * kSHid, s->st) ||
        launch_gemm_bf16(s->Hb, kSHid, s->w3t, kSHid, s->p + kOffB3, s->Y, kSOut, nn, kSOut,
                         kSHid, s->d_err, s->st) ||
        launch_surr_calib(s->xs + r0 * kSIn, s->ts + r0 * kSM, s->Y, kSOut, nr, s->mu32,
                          res + r0, err + r0, s->st))
      e = cudaGetLastError();
  }
  std::vector<float> hr(n), he(n);
  if (e == cudaSuccess) e = cudaMemcpyAsync(hr.data(), res, n * sizeof(float), cudaMemcpyDeviceToHost, s->st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(he.data(), err, n * sizeof(float), cudaMemcpyDeviceToHost, s->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->st);
  cudaFree(res);
  cudaFree(err);
  if (e != cudaSuccess) return cuda_fail(e, "calibrate_error");
  const int rc = surr_read_err(s);
  if (rc) return rc;
  // the smallest residual of a row beyond target bounds the tolerance
  float bound = INFINITY;
  size_t ok = 0;
  for (size_t i = 0; i < n; i++) {
    const bool good = he[i] <= (float)target;  // false for NaN
    ok += good;
    if (!good) bound = std::min(bound, std::isnan(hr[i]) ? -INFINITY : hr[i]);
  }
  size_t keep = 0;
  for (size_t i = 0; i < n; i++) keep += hr[i] < bound;  // false for NaN
  s->tol = std::isinf(bound) && bound > 0 ? INFINITY : std::nextafter(bound, -INFINITY);
  if (tol_out) *tol_out = s->tol;
  if (kept) *kept = (double)keep / (double)n;
  if (within) *within = (double)ok / (double)n;
  return EPREM_GPU_OK;
}

extern "C" int eprem_gpu_surrogate_set_tolerance(eprem_gpu_surrogate *s, double tol) {
  if (!s) return fail(EPREM_GPU_ERR_ARG, "null surrogate");
  s->tol = (float)tol;
  return EPREM_GPU_OK;
}

// Node phase of the split and surrogate forms, one EP sub-step.
int eprem::split_node_phase(eprem_gpu_run *r) {
  const size_t rows = r->sn() * r->dims.num_energies;
  RunView change_only = r->v;
  change_only.use_focus = 0;
  if (r->node_mode == EPREM_NODE_PHASE_SPLIT) {
    if (launch_split_focus_relax(r->v, 0, rows, nullptr, r->stream, &r->launches))
      return EPREM_GPU_ERR_CUDA;
  } else {
    eprem_gpu_surrogate *s = r->surr;
    const cudaStream_t st = r->stream;
    for (size_t row0 = 0; row0 < rows; row0 += s->R) {
      const size_t nr = std::min(s->R, rows - row0);
      const int n = (int)nr;
      if (launch_surr_features(r->v, row0, nr, s->X, st, &r->launches) ||
          launch_gemm_bf16(s->X, kSIn, s->w1t, kSIn, s->p + kOffB1, s->Z, kSHid, n, kSHid, kSIn,
                           s->d_err, st) ||
          launch_gelu_bf16(s->Z, s->Ha, nr * kSHid, st) ||
          launch_gemm_bf16(s->Ha, kSHid, s->w2t, kSHid, s->p + kOffB2, s->Z, kSHid, n, kSHid,
                           kSHid, s->d_err, st) ||
          launch_gelu_bf16(s->Z, s->Hb, nr * kSHid, st) ||
          launch_gemm_bf16(s->Hb, kSHid, s->w3t, kSHid, s->p + kOffB3, s->Y, kSOut, n, kSOut,
                           kSHid, s->d_err, st) ||
          launch_surr_apply(r->v, row0, nr, s->Y, kSOut, s->tol, r->d_reject, r->d_surr_counts,
                            st, &r->launches) ||
          launch_split_focus_relax(r->v, row0, nr, r->d_reject, st, &r->launches))
        return EPREM_GPU_ERR_CUDA;
      r->launches += 5;  // the three GEMMs and two GELU kernels
    }
  }
  if (r->v.use_change && launch_node32(change_only, r->nplan, r->stream, &r->launches))
    return EPREM_GPU_ERR_CUDA;
  return EPREM_GPU_OK;
}

extern "C" int eprem_gpu_set_node_phase(eprem_gpu_run *r, int mode, eprem_gpu_surrogate *s) {
  if (!r) return fail(EPREM_GPU_ERR_ARG, "null run");
  if (mode == EPREM_NODE_PHASE_REFERENCE) {
    r->node_mode = mode;
    r->v.relax_in_stream = 1;
    r->surr = nullptr;
    return EPREM_GPU_OK;
  }
  if (mode != EPREM_NODE_PHASE_SPLIT && mode != EPREM_NODE_PHASE_SURROGATE &&
      mode != EPREM_NODE_PHASE_SURROGATE_FOCUS)
    return fail(EPREM_GPU_ERR_ARG, "unknown node phase");
  const int rc = surr_check_run(r);
  if (rc) return rc;
  const bool surrogate = mode != EPREM_NODE_PHASE_SPLIT;
  if (surrogate) {
    if (!s) return fail(EPREM_GPU_ERR_ARG, "the surrogate form needs a surrogate");
    if (s->device != r->device) return fail(EPREM_GPU_ERR_ARG, "surrogate on another device");
    if (!r->d_surr_counts) CK(cudaMalloc(&r->d_surr_counts, 2 * sizeof(unsigned long long)));
    if (!r->d_reject) CK(cudaMalloc(&r->d_reject, s->R));
    CK(cudaMemsetAsync(r->d_surr_counts, 0, 2 * sizeof(unsigned long long), r->stream));
    CK(cudaStreamSynchronize(r->stream));
  }
  r->node_mode = mode;
  r->v.relax_in_stream = mode == EPREM_NODE_PHASE_SURROGATE_FOCUS ? 1 : 0;
  r->surr = surrogate ? s : nullptr;
  return EPREM_GPU_OK;
}

extern "C" int eprem_gpu_surrogate_counts(eprem_gpu_run *r, uint64_t *kept, uint64_t *fallback) {
  if (!r || !kept || !fallback) return fail(EPREM_GPU_ERR_ARG, "null argument");
  unsigned long long h[2] = {0, 0};
  if (r->d_surr_counts) {
    CK(cudaMemcpyAsync(h, r->d_surr_counts, sizeof(h), cudaMemcpyDeviceToHost, r->stream));
    CK(cudaStreamSynchronize(r->stream));
  }
  *kept = h[0];
  *fallback = h[1];
  if (r->surr) return surr_read_err(r->surr);
  return EPREM_GPU_OK;
}
