// ensemble.cu -- autotuning of the streaming shape and ensembles of runs
// stepped by one CUDA-graph launch (no counterpart in the reference, which
// runs one simulation per process).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "run.h"

using namespace eprem;

// ---- autotuner ---------------------------------------------------------------
// Times the FP32 streaming-kernel shapes on a scratch copy of the run's first
// streams (the kernel that takes 90 % of a step) and keeps the fastest.  The
// copy has its own status block, so the run's statistics are untouched.
namespace {
constexpr int kTuneVariants[] = {5, 4, 3};

int tune_stream(eprem_gpu_run *r, int *chosen) {
  const eprem_params_t &p = r->params;
  CK(cudaStreamSynchronize(r->stream));
  int rc = launch_geometry(r->v, r->stream, r->norm_radius, r->neg_beta, p.mfp_type,
                           p.mfp_type == 2 ? p.mfp_b_power : p.mfp_radial_power, p.mhd_bs_au,
                           &r->launches);
  if (rc) return cuda_fail(cudaGetLastError(), "autotune geometry launch");
  if (r->d_scoef && launch_stream2_coef(r->v, r->stream, &r->launches))
    return cuda_fail(cudaGetLastError(), "autotune coefficient launch");
  const int S_sub = r->dims.num_streams < 96 ? r->dims.num_streams : 96;
  const size_t n = (size_t)S_sub * r->dims.num_nodes * r->dims.num_energies * r->dims.num_mu;
  const size_t nrows = n / r->dims.num_mu;
  void *f = nullptr;
  short *fx = nullptr;  // the copy's row exponents
  DevStatus *st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaMalloc(&f, n * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&fx, nrows * sizeof(short));
  if (e == cudaSuccess) e = cudaMalloc(&st, sizeof(DevStatus));
  if (e == cudaSuccess) e = cudaMemsetAsync(st, 0, sizeof(DevStatus), r->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(f, r->d_f, n * sizeof(float), cudaMemcpyDeviceToDevice, r->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(fx, r->d_fexp, nrows * sizeof(short), cudaMemcpyDeviceToDevice,
                        r->stream);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  RunView v = r->v;
  v.S = S_sub;
  v.f = f;
  v.fexp = fx;
  v.status = st;
  float best = -1.f;
  int best_variant = 0;
  StreamPlan best_plan{};
  uint64_t dummy = 0;
  for (int variant : kTuneVariants) {
    if (e != cudaSuccess) break;
    StreamPlan pl{};
    if (plan_stream(EPREM_FP32, r->dims.num_nodes, r->dims.num_mu, r->m0, variant, &pl)) continue;
    if (launch_stream(v, pl, r->m0, r->stream, &dummy)) {  // warm-up
      e = cudaGetLastError();
      break;
    }
    cudaEventRecord(e0, r->stream);
    for (int k = 0; k < 2; k++) launch_stream(v, pl, r->m0, r->stream, &dummy);
    cudaEventRecord(e1, r->stream);
    e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e == cudaSuccess && (best < 0.f || ms < best)) {
      best = ms;
      best_variant = variant;
      best_plan = pl;
    }
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(r->stream);
  cudaFree(f);
  cudaFree(fx);
  cudaFree(st);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (e != cudaSuccess) return cuda_fail(e, "autotune");
  if (best_variant) {
    r->splan = best_plan;
    r->params.stream_variant = best_variant;
  }
  *chosen = r->params.stream_variant;
  return EPREM_GPU_OK;
}
}  // namespace

extern "C" int eprem_gpu_autotune(eprem_gpu_run *r, int *chosen_variant) {
  if (!r || !chosen_variant) return fail(EPREM_GPU_ERR_ARG, "null argument");
  if (r->dims.precision != EPREM_FP32 || !r->v.use_stream) {
    *chosen_variant = r->params.stream_variant;  // one shape only
    return EPREM_GPU_OK;
  }
  return tune_stream(r, chosen_variant);
}

extern "C" int eprem_gpu_set_stream_variant(eprem_gpu_run *r, int variant) {
  if (!r) return fail(EPREM_GPU_ERR_ARG, "null run");
  StreamPlan pl{};
  if (plan_stream(r->dims.precision, r->dims.num_nodes, r->dims.num_mu, r->m0, variant, &pl))
    return fail(EPREM_GPU_ERR_ARG, "streaming variant does not fit this run's sizes");
  r->splan = pl;
  r->params.stream_variant = variant;
  return EPREM_GPU_OK;
}

// ---- ensembles -------------------------------------------------------------
// Independent runs stepped together.  The first eprem_gpu_ensemble_step
// captures one driver step of every run (moveNodes, updateMhd at t + tDel,
// updateEnergeticParticles, t += tDel) into one CUDA graph, the runs on
// serial chains (one by default, or one branch per run) between a fork and a
// join on the ensemble's stream; every step
// after that is one graph launch.  Each run's time lives on the device so
// the replayed graph advances it.
struct eprem_gpu_ensemble {
  std::vector<eprem_gpu_run *> runs;
  int device = 0;
  cudaStream_t origin = nullptr;
  cudaEvent_t fork = nullptr;
  std::vector<cudaEvent_t> joins;
  double *d_time = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<uint64_t> launches_per_step;
  int chains = 1;  // serial chains side by side; 0: one branch per run
};

static void ensemble_drop_graph(eprem_gpu_ensemble *e) {
  if (e->exec) cudaGraphExecDestroy(e->exec);
  if (e->graph) cudaGraphDestroy(e->graph);
  e->exec = nullptr;
  e->graph = nullptr;
}

extern "C" int eprem_gpu_ensemble_destroy(eprem_gpu_ensemble *e) {
  if (!e) return EPREM_GPU_OK;
  if (e->origin) cudaStreamSynchronize(e->origin);
  ensemble_drop_graph(e);
  for (cudaEvent_t ev : e->joins) cudaEventDestroy(ev);
  if (e->fork) cudaEventDestroy(e->fork);
  cudaFree(e->d_time);
  if (e->origin) cudaStreamDestroy(e->origin);
  delete e;
  return EPREM_GPU_OK;
}

extern "C" int eprem_gpu_ensemble_create(eprem_gpu_run *const *runs, int n,
                                         eprem_gpu_ensemble **out) {
  if (!runs || !out || n <= 0) return fail(EPREM_GPU_ERR_ARG, "ensemble needs runs");
  *out = nullptr;
  int dev = -1;
  CK(cudaGetDevice(&dev));
  for (int i = 0; i < n; i++) {
    if (!runs[i]) return fail(EPREM_GPU_ERR_ARG, "null run in ensemble");
    if (runs[i]->device != dev)
      return fail(EPREM_GPU_ERR_ARG, "ensemble runs must live on the current device");
    if (runs[i]->mas_ready)
      return fail(EPREM_GPU_ERR_UNSUPPORTED,
                  "ensemble steps use the analytic background; MAS runs step one by one");
    if (runs[i]->surr)
      return fail(EPREM_GPU_ERR_UNSUPPORTED, "surrogate-form runs step one by one");
    if (runs[i]->shell_on)
      return fail(EPREM_GPU_ERR_UNSUPPORTED, "runs with shell diffusion step one by one");
    for (int j = 0; j < i; j++)
      if (runs[j] == runs[i]) return fail(EPREM_GPU_ERR_ARG, "run listed twice in ensemble");
  }
  auto *e = new eprem_gpu_ensemble();
  e->runs.assign(runs, runs + n);
  e->device = dev;
  e->joins.assign(n, nullptr);
  e->launches_per_step.assign(n, 0);
  cudaError_t err = cudaStreamCreateWithFlags(&e->origin, cudaStreamNonBlocking);
  if (err == cudaSuccess) err = cudaEventCreateWithFlags(&e->fork, cudaEventDisableTiming);
  for (int i = 0; i < n && err == cudaSuccess; i++)
    err = cudaEventCreateWithFlags(&e->joins[i], cudaEventDisableTiming);
  if (err == cudaSuccess) err = cudaMalloc(&e->d_time, n * sizeof(double));
  if (err == cudaSuccess) err = cudaMemsetAsync(e->d_time, 0, n * sizeof(double), e->origin);
  if (err == cudaSuccess) err = cudaStreamSynchronize(e->origin);
  if (err != cudaSuccess) {
    eprem_gpu_ensemble_destroy(e);
    return cuda_fail(err, "eprem_gpu_ensemble_create");
  }
  *out = e;
  return EPREM_GPU_OK;
}

extern "C" int eprem_gpu_ensemble_set_time(eprem_gpu_ensemble *e, const double *t_global) {
  if (!e || !t_global) return fail(EPREM_GPU_ERR_ARG, "null argument");
  CK(cudaMemcpyAsync(e->d_time, t_global, e->runs.size() * sizeof(double),
                     cudaMemcpyHostToDevice, e->origin));
  CK(cudaStreamSynchronize(e->origin));
  return EPREM_GPU_OK;
}

extern "C" int eprem_gpu_ensemble_get_time(eprem_gpu_ensemble *e, double *t_global) {
  if (!e || !t_global) return fail(EPREM_GPU_ERR_ARG, "null argument");
  CK(cudaMemcpyAsync(t_global, e->d_time, e->runs.size() * sizeof(double),
                     cudaMemcpyDeviceToHost, e->origin));
  CK(cudaStreamSynchronize(e->origin));
  return EPREM_GPU_OK;
}

extern "C" int eprem_gpu_ensemble_autotune(eprem_gpu_ensemble *e, int *chosen_variants) {
  if (!e) return fail(EPREM_GPU_ERR_ARG, "null ensemble");
  // size class: precision, mu bin and cluster shape of the default plan
  std::vector<std::pair<std::vector<int>, int>> classes;  // key -> variant
  for (size_t i = 0; i < e->runs.size(); i++) {
    eprem_gpu_run *r = e->runs[i];
    StreamPlan key{};
    plan_stream(r->dims.precision, r->dims.num_nodes, r->dims.num_mu, r->m0, 0, &key);
    const std::vector<int> k = {r->dims.precision, key.mmax, key.cluster, key.threads,
                                r->dims.num_mu, r->m0};
    int variant = -1;
    for (auto &c : classes)
      if (c.first == k) variant = c.second;
    int rc;
    if (variant < 0) {
      rc = eprem_gpu_autotune(r, &variant);
      if (rc) return rc;
      classes.push_back({k, variant});
    } else {
      rc = eprem_gpu_set_stream_variant(r, variant);
      if (rc) return rc;
    }
    if (chosen_variants) chosen_variants[i] = variant;
  }
  ensemble_drop_graph(e);  // plans changed: capture again on the next step
  return EPREM_GPU_OK;
}

static int ensemble_capture(eprem_gpu_ensemble *e) {
  const int n = (int)e->runs.size();
  std::vector<bool> saved(n);
  for (int i = 0; i < n; i++) saved[i] = e->runs[i]->timing;
  CK(cudaStreamBeginCapture(e->origin, cudaStreamCaptureModeRelaxed));
  int rc = EPREM_GPU_OK;
  cudaError_t err = cudaEventRecord(e->fork, e->origin);
  // chain of each run: largest run first onto the chain with the fewest cells
  const int nch = (e->chains <= 0 || e->chains > n) ? n : e->chains;
  std::vector<int> order(n), chain_of(n, 0);
  for (int i = 0; i < n; i++) order[i] = i;
  auto cells = [&](int i) { return (double)e->runs[i]->cells(); };
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cells(a) > cells(b); });
  std::vector<double> load(nch, 0.0);
  std::vector<int> last(nch, -1);  // last run on each chain so far
  for (int i : order) {
    const int c = (int)(std::min_element(load.begin(), load.end()) - load.begin());
    chain_of[i] = c;
    load[c] += cells(i);
  }
  for (int k = 0; k < n && err == cudaSuccess && rc == EPREM_GPU_OK; k++) {
    const int i = order[k];
    eprem_gpu_run *r = e->runs[i];
    r->timing = false;  // no event bookkeeping inside a graph
    const uint64_t l0 = r->launches;
    const int prev = last[chain_of[i]];
    err = cudaStreamWaitEvent(r->stream, prev < 0 ? e->fork : e->joins[prev], 0);
    if (err != cudaSuccess) break;
    last[chain_of[i]] = i;
    const double td = r->params.t_del;
    if (launch_move_nodes(r->v, td, r->stream, &r->launches) ||
        launch_update_mhd(r->v, r->mhd, td, r->stream, &r->launches, e->d_time + i)) {
      err = cudaGetLastError();
      break;
    }
    rc = eprem_gpu_update_energetic_particles(r, 0.0);
    if (rc) break;
    if (launch_advance_time(e->d_time + i, td, r->stream, &r->launches)) {
      err = cudaGetLastError();
      break;
    }
    e->launches_per_step[i] = r->launches - l0;
    r->launches = l0;  // counted again at every replay
    err = cudaEventRecord(e->joins[i], r->stream);
  }
  for (int c = 0; c < nch && err == cudaSuccess; c++)
    if (last[c] >= 0) err = cudaStreamWaitEvent(e->origin, e->joins[last[c]], 0);
  for (int i = 0; i < n; i++) e->runs[i]->timing = saved[i];
  cudaGraph_t g = nullptr;
  const cudaError_t end = cudaStreamEndCapture(e->origin, &g);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (err == cudaSuccess) err = end;
  if (err == cudaSuccess) err = cudaGraphInstantiate(&e->exec, g, 0);
  if (err != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    e->exec = nullptr;
    return cuda_fail(err, "ensemble step capture");
  }
  e->graph = g;
  return EPREM_GPU_OK;
}

extern "C" int eprem_gpu_ensemble_set_chains(eprem_gpu_ensemble *e, int chains) {
  if (!e) return fail(EPREM_GPU_ERR_ARG, "null ensemble");
  if (chains < 0) return fail(EPREM_GPU_ERR_ARG, "chains must be >= 0");
  if (chains != e->chains) {
    if (e->origin) CK(cudaStreamSynchronize(e->origin));
    ensemble_drop_graph(e);
    e->chains = chains;
  }
  return EPREM_GPU_OK;
}

extern "C" int eprem_gpu_ensemble_step(eprem_gpu_ensemble *e) {
  if (!e) return fail(EPREM_GPU_ERR_ARG, "null ensemble");
  for (eprem_gpu_run *r : e->runs)  // switched on after the ensemble was made
    if (r->shell_on)
      return fail(EPREM_GPU_ERR_UNSUPPORTED, "runs with shell diffusion step one by one");
  if (!e->exec) {
    const int rc = ensemble_capture(e);
    if (rc) return rc;
  }
  CK(cudaGraphLaunch(e->exec, e->origin));
  for (size_t i = 0; i < e->runs.size(); i++) e->runs[i]->launches += e->launches_per_step[i];
  return EPREM_GPU_OK;
}

extern "C" int eprem_gpu_ensemble_synchronize(eprem_gpu_ensemble *e) {
  if (!e) return fail(EPREM_GPU_ERR_ARG, "null ensemble");
  CK(cudaStreamSynchronize(e->origin));
  for (eprem_gpu_run *r : e->runs) {
    const int rc = check_status(r, false, nullptr);
    if (rc) return rc;
  }
  return EPREM_GPU_OK;
}

extern "C" void *eprem_gpu_ensemble_stream(eprem_gpu_ensemble *e) {
  return e ? (void *)e->origin : nullptr;
}

