// ensemble.cu -- autotuning of the streaming shape and ensembles of runs
// stepped by one CUDA-graph launch (no counterpart in the reference, which
// runs one simulation per process).
#include <algorithm>
#include <cstdio>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "run.h"

using namespace eprem;

// ---- autotuner ---------------------------------------------------------------
// Times the FP32 streaming kernels on a scratch copy of the run's first
// streams (the kernel that takes 90 % of a step) and keeps the fastest: every
// kind that fits the run (mirrored, compile-time guards, packed, scalar) in every CTA
// shape of its mu bin (threads per CTA, list nodes per thread, and so the
// cluster size for the run's stream length).  The copy has its own status
// block, so the run's statistics are untouched.
namespace {
constexpr int kTuneKinds[] = {7, 6, 5, 4, 3};

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
  std::vector<int> variants;
  for (int shape = 1; shape <= stream2_shape_count(r->dims.num_mu); ++shape)
    for (int kind : kTuneKinds) variants.push_back(kind + 8 * shape);
  for (int variant : variants) {
    if (e != cudaSuccess) break;
    StreamPlan pl{};
    if (plan_stream(EPREM_FP32, r->dims.num_nodes, r->dims.num_mu, r->m0, variant,
                    r->v.use_bc != 0, &pl))
      continue;
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

extern "C" int eprem_gpu_plan_stream(int num_nodes, int num_mu, int m0, int precision,
                                     int variant, int seed_boundary, int out[6]) {
  if (!out || num_nodes < 3 || num_mu < 2 || num_mu > 64 || m0 < 0 || m0 > num_mu)
    return fail(EPREM_GPU_ERR_ARG, "bad sizes");
  StreamPlan p{};
  if (plan_stream(precision, num_nodes, num_mu, m0, variant, seed_boundary != 0, &p))
    return fail(EPREM_GPU_ERR_ARG, "no streaming kernel fits these sizes");
  const bool s2 = p.reg_coef == 2;
  out[0] = !s2 ? 0 : p.mirror ? 5 + p.mirror : !p.packed ? 3 : p.filled ? 5 : 4;
  out[1] = p.mmax;
  out[2] = p.threads;
  out[3] = s2 ? p.npt : 1;
  out[4] = p.cluster;
  out[5] = p.threads * (s2 ? p.npt : 1) * p.cluster;
  return EPREM_GPU_OK;
}

extern "C" const char *eprem_gpu_stream_kernel(eprem_gpu_run *r) {
  if (!r) return "";
  const StreamPlan &p = r->splan;
  char buf[96];
  if (p.reg_coef != 2)
    snprintf(buf, sizeof(buf), "k_stream<%d> cluster %d", p.mmax, p.cluster);
  else
    snprintf(buf, sizeof(buf), "%s<%d,%d,%d> cluster %d",
             p.mirror ? "k_stream2_mirror" : p.packed ? "k_stream2_pairs" : "k_stream2", p.mmax,
             p.threads, p.npt, p.cluster);
  r->skernel = buf;
  return r->skernel.c_str();
}

extern "C" int eprem_gpu_set_stream_variant(eprem_gpu_run *r, int variant) {
  if (!r) return fail(EPREM_GPU_ERR_ARG, "null run");
  StreamPlan pl{};
  if (plan_stream(r->dims.precision, r->dims.num_nodes, r->dims.num_mu, r->m0, variant,
                  r->v.use_bc != 0, &pl))
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
  int chains = -1;  // < 0 lock-step with merged streaming; 0 one branch per run; k serial chains
  // lock-step: the slab lists of the merged streaming launches
  std::vector<int4 *> d_items;
};

static void ensemble_drop_graph(eprem_gpu_ensemble *e) {
  if (e->exec) cudaGraphExecDestroy(e->exec);
  if (e->graph) cudaGraphDestroy(e->graph);
  e->exec = nullptr;
  e->graph = nullptr;
  for (int4 *p : e->d_items) cudaFree(p);
  e->d_items.clear();
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
    if (runs[i]->shell_on || runs[i]->drift_on)
      return fail(EPREM_GPU_ERR_UNSUPPORTED,
                  "runs with shell diffusion or drift step one by one");
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
    plan_stream(r->dims.precision, r->dims.num_nodes, r->dims.num_mu, r->m0, 0,
                r->v.use_bc != 0, &key);
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

// Lock-step capture: every run's per-call set-up, then EP sub-step by EP
// sub-step the streaming of all runs -- one launch per group of runs that
// share a packed streaming kernel (mu bin, CTA shape, cluster size, guards),
// the group's (run, stream, energy) slabs ordered by their estimated work,
// longest first, so the slabs of small runs fill the tails of large ones --
// and the node phases -- one focusing and one change launch per group of
// runs of one mu count over all their row and node blocks, the other runs'
// own launches; all on the ensemble's stream.  Each slab and
// row is computed by the same code as in a run's own update: the results are
// the runs' own, bit for bit.  Needs the same numEpSteps in every run.
namespace {
struct S2Group {
  StreamPlan plan;
  std::vector<int> runs;  // ensemble indices
};
bool same_plan(const StreamPlan &a, const StreamPlan &b) {
  return a.mmax == b.mmax && a.threads == b.threads && a.npt == b.npt && a.cluster == b.cluster &&
         a.packed == b.packed && a.filled == b.filled && a.reg_coef == b.reg_coef &&
         a.mirror == b.mirror;
}
}  // namespace

static int ensemble_capture_lockstep(eprem_gpu_ensemble *e) {
  const int n = (int)e->runs.size();
  // the slabs' work estimates need each run's stream geometry: one geometry
  // pass (its values are the ones the step itself forms, up to the step's
  // node motion) before the capture
  std::vector<std::vector<double>> ds_min(n);
  std::vector<std::vector<int>> list_size(n);
  for (int i = 0; i < n; i++) {
    eprem_gpu_run *r = e->runs[i];
    const eprem_params_t &p = r->params;
    if (launch_geometry(r->v, r->stream, r->norm_radius, r->neg_beta, p.mfp_type,
                        p.mfp_type == 2 ? p.mfp_b_power : p.mfp_radial_power, p.mhd_bs_au,
                        &r->launches))
      return cuda_fail(cudaGetLastError(), "ensemble geometry launch");
    const int S = r->dims.num_streams;
    ds_min[i].resize(S);
    list_size[i].resize(S);
    CK(cudaMemcpyAsync(ds_min[i].data(), r->d_ds_min, S * sizeof(double),
                       cudaMemcpyDeviceToHost, r->stream));
    CK(cudaMemcpyAsync(list_size[i].data(), r->d_list_size, S * sizeof(int),
                       cudaMemcpyDeviceToHost, r->stream));
    CK(cudaStreamSynchronize(r->stream));
  }
  std::vector<S2Group> groups;
  std::vector<int> solo;
  for (int i = 0; i < n; i++) {
    eprem_gpu_run *r = e->runs[i];
    const StreamPlan &pl = r->splan;
    if (!r->v.use_stream || pl.reg_coef != 2 || !pl.packed) {
      solo.push_back(i);
      continue;
    }
    bool found = false;
    for (auto &g : groups)
      if (same_plan(g.plan, pl) && (int)g.runs.size() < kMultiRuns) {
        g.runs.push_back(i);
        found = true;
        break;
      }
    if (!found) groups.push_back({pl, {i}});
  }
  std::vector<MultiRunViews> views(groups.size());
  std::vector<int> n_items(groups.size());
  for (size_t gi = 0; gi < groups.size(); gi++) {
    std::vector<std::pair<double, int4>> items;
    for (int j = 0; j < (int)groups[gi].runs.size(); j++) {
      eprem_gpu_run *r = e->runs[groups[gi].runs[j]];
      views[gi].v[j] = r->v;
      views[gi].m0[j] = r->m0;
      const double dt = r->v.dt;
      for (int s = 0; s < r->dims.num_streams; s++)
        for (int en = 0; en < r->dims.num_energies; en++) {
          const double dtMin = 0.4 * ds_min[groups[gi].runs[j]][s] * r->h_ec[en].vgrid_i;
          const double nst = dtMin > 0.0 ? floor(dt / dtMin + 1.0) : 1.0;
          const double cost = nst * list_size[groups[gi].runs[j]][s] * r->dims.num_mu;
          items.push_back({cost, make_int4(j, s, en, 0)});
        }
    }
    std::stable_sort(items.begin(), items.end(),
                     [](const auto &a, const auto &b) { return a.first > b.first; });
    std::vector<int4> flat(items.size());
    for (size_t k = 0; k < items.size(); k++) flat[k] = items[k].second;
    int4 *d = nullptr;
    CK(cudaMalloc(&d, flat.size() * sizeof(int4)));
    e->d_items.push_back(d);
    CK(cudaMemcpy(d, flat.data(), flat.size() * sizeof(int4), cudaMemcpyHostToDevice));
    n_items[gi] = (int)flat.size();
  }
  // node phases: runs of one mu count in the plain form, focusing and change
  // both on, in two launches per sub-step over all their (run, block) items
  struct NodeGroup {
    int M;
    std::vector<int> runs;
    NodeRunViews views;
  };
  std::vector<NodeGroup> ngroups;
  std::vector<char> node_grouped(n, 0);
  for (int i = 0; i < n; i++) {
    eprem_gpu_run *r = e->runs[i];
    if (r->node_mode != EPREM_NODE_PHASE_REFERENCE || !r->nplan.fast32 || !r->v.use_focus ||
        !r->v.use_change || r->shell_on || r->drift_on)
      continue;
    NodeGroup *grp = nullptr;
    for (auto &ng : ngroups)
      if (ng.M == r->dims.num_mu && (int)ng.runs.size() < kMultiRuns) grp = &ng;
    if (!grp) {
      ngroups.push_back(NodeGroup{});
      grp = &ngroups.back();
      grp->M = r->dims.num_mu;
    }
    grp->runs.push_back(i);
  }
  for (auto &ng : ngroups) {
    ng.views.n = 0;
    if (ng.runs.size() < 2) continue;  // a lone run keeps its own launches
    ng.views.n = (int)ng.runs.size();
    ng.views.foff[0] = ng.views.coff[0] = 0;
    for (int j = 0; j < ng.views.n; j++) {
      eprem_gpu_run *r = e->runs[ng.runs[j]];
      ng.views.v[j] = r->v;
      int nf = 0, nc = 0;
      node32_blocks(r->v, &nf, &nc);
      ng.views.foff[j + 1] = ng.views.foff[j] + nf;
      ng.views.coff[j + 1] = ng.views.coff[j] + nc;
      node_grouped[ng.runs[j]] = 1;
    }
  }
  std::vector<bool> saved(n);
  std::vector<cudaStream_t> own(n);
  for (int i = 0; i < n; i++) {
    saved[i] = e->runs[i]->timing;
    own[i] = e->runs[i]->stream;
    e->runs[i]->timing = false;       // no event bookkeeping inside a graph
    e->runs[i]->stream = e->origin;   // every launch on the ensemble's stream
  }
  std::vector<uint64_t> l0(n);
  for (int i = 0; i < n; i++) l0[i] = e->runs[i]->launches;
  CK(cudaStreamBeginCapture(e->origin, cudaStreamCaptureModeRelaxed));
  int rc = EPREM_GPU_OK;
  cudaError_t err = cudaSuccess;
  const int nsub = e->runs[0]->params.num_ep_steps;
  for (int i = 0; i < n && !rc && err == cudaSuccess; i++) {
    eprem_gpu_run *r = e->runs[i];
    const double td = r->params.t_del;
    if (launch_move_nodes(r->v, td, r->stream, &r->launches) ||
        launch_update_mhd(r->v, r->mhd, td, r->stream, &r->launches, e->d_time + i))
      err = cudaGetLastError();
    else
      rc = ep_begin(r, r->v);
  }
  for (int step = 0; step < nsub && !rc && err == cudaSuccess; step++) {
    for (size_t gi = 0; gi < groups.size() && !rc; gi++)
      if (launch_stream2_multi(groups[gi].plan, views[gi], e->d_items[gi], n_items[gi],
                               e->origin, &e->runs[groups[gi].runs[0]]->launches))
        err = cudaGetLastError();
    for (int i : solo)
      if (!rc && err == cudaSuccess) rc = ep_stream_phase(e->runs[i], e->runs[i]->v);
    for (auto &ng : ngroups)
      if (ng.views.n && !rc && err == cudaSuccess &&
          launch_node32_multi(e->runs[ng.runs[0]]->nplan, ng.views, e->origin,
                              &e->runs[ng.runs[0]]->launches))
        err = cudaGetLastError();
    for (int i = 0; i < n && !rc && err == cudaSuccess; i++)
      if (!node_grouped[i]) rc = ep_node_phase(e->runs[i], e->runs[i]->v);
  }
  for (int i = 0; i < n && !rc && err == cudaSuccess; i++) {
    eprem_gpu_run *r = e->runs[i];
    if (launch_advance_time(e->d_time + i, r->params.t_del, r->stream, &r->launches))
      err = cudaGetLastError();
  }
  for (int i = 0; i < n; i++) {
    e->runs[i]->timing = saved[i];
    e->runs[i]->stream = own[i];
    e->launches_per_step[i] = e->runs[i]->launches - l0[i];
    e->runs[i]->launches = l0[i];  // counted again at every replay
  }
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

static int ensemble_capture(eprem_gpu_ensemble *e) {
  if (e->chains < 0) {
    bool same = true;
    for (eprem_gpu_run *r : e->runs)
      same = same && r->params.num_ep_steps == e->runs[0]->params.num_ep_steps;
    if (same) return ensemble_capture_lockstep(e);
  }
  const int n = (int)e->runs.size();
  std::vector<bool> saved(n);
  for (int i = 0; i < n; i++) saved[i] = e->runs[i]->timing;
  CK(cudaStreamBeginCapture(e->origin, cudaStreamCaptureModeRelaxed));
  int rc = EPREM_GPU_OK;
  cudaError_t err = cudaEventRecord(e->fork, e->origin);
  // chain of each run: largest run first onto the chain with the fewest cells
  const int nch = (e->chains == 0 || e->chains > n) ? n : (e->chains < 0 ? 1 : e->chains);
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
  if (chains < 0) chains = -1;
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
    if (r->shell_on || r->drift_on)
      return fail(EPREM_GPU_ERR_UNSUPPORTED,
                  "runs with shell diffusion or drift step one by one");
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

