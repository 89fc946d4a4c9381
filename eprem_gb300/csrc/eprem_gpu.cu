// eprem_gpu.cu -- the C ABI of include/eprem_gpu.h.
//
// Owns the device state of a run and sequences the kernels the way the
// reference's entry points sequence their loops:
//   updateEnergeticParticles (src/energeticParticles.c:70-203)
//     geometry once per call (positions are fixed during the call), then per
//     EP sub-step: streaming (+ seed check) over all (stream, energy) slabs,
//     then focusing + change over all nodes;
//   updateMhd (src/flow.c:36-154), moveNodes (src/simCore.c:737-785).
// Device failures (NaN/Inf, ds <= 0, sub-cycle cap) land in a status block
// that the synchronising calls read and turn into the reference's panic text.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"
#include "kernels.h"

using namespace eprem;

namespace {
thread_local std::string g_last_error;

int fail(int code, const std::string &msg) {
  g_last_error = msg;
  return code;
}

int cuda_fail(cudaError_t e, const char *what) {
  return fail(EPREM_GPU_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(call)                                   \
  do {                                             \
    cudaError_t _e = (call);                       \
    if (_e != cudaSuccess) return cuda_fail(_e, #call); \
  } while (0)

const double kEfac = kMev / (kMp * kC * kC);
}  // namespace

struct eprem_gpu_run {
  eprem_dims_t dims;
  eprem_params_t params;
  int device = 0;
  cudaStream_t stream = nullptr;
  RunView v{};
  MhdParams mhd{};
  StreamPlan splan{};
  NodePlan nplan{};
  int m0 = 0;
  double norm_radius = 0, neg_beta = 0;
  void *d_f = nullptr;
  double *d_nodes = nullptr, *d_mugrid = nullptr;
  float *d_mugrid32 = nullptr;
  NodeCoef32 *d_coef32 = nullptr;
  EnergyConsts *d_ec = nullptr;
  int *d_list = nullptr, *d_list_size = nullptr;
  double *d_ds_i = nullptr, *d_ds_min = nullptr, *d_seed_radial = nullptr, *d_mfp_node = nullptr;
  DevStatus *d_status = nullptr, *h_status = nullptr;
  double *d_stage = nullptr;
  size_t stage_elems = 0;
  double *d_flux = nullptr;
  uint64_t launches = 0;
  // optional per-launch timing: events recorded around each kernel launch
  bool timing = false;
  std::vector<cudaEvent_t> ev_pool;
  std::vector<std::pair<int, int>> ev_pending;  // (kind, index of start event)
  size_t ev_used = 0;
  // MAS background: device copies of the loaded time slices
  int node_mode = 0;                       // EPREM_NODE_PHASE_*
  struct eprem_gpu_surrogate *surr = nullptr;
  unsigned long long *d_surr_counts = nullptr;  // [kept, fallback] rows
  uint8_t *d_reject = nullptr;
  bool mas_ready = false;  // eprem_gpu_mas_init done
  bool mas_on = false, mas_selected = false;  // updateMhd uses MAS; slots chosen
  std::vector<std::vector<void *>> mas_allocs;
  std::vector<MasSlotDev> mas_slots;
  std::vector<char> mas_loaded;
  MasView mv{};
  size_t cells() const {
    return (size_t)dims.num_streams * dims.num_nodes * dims.num_energies * dims.num_mu;
  }
  size_t sn() const { return (size_t)dims.num_streams * dims.num_nodes; }
};

// Runs one launch helper, bracketed by events when timing is on.
template <typename Fn>
static int timed(eprem_gpu_run *r, int kind, Fn &&launch) {
  if (!r->timing) return launch();
  if (r->ev_used + 2 > r->ev_pool.size()) {
    for (int i = 0; i < 64; i++) {
      cudaEvent_t ev;
      if (cudaEventCreate(&ev) != cudaSuccess) return EPREM_GPU_ERR_CUDA;
      r->ev_pool.push_back(ev);
    }
  }
  const size_t i0 = r->ev_used;
  r->ev_used += 2;
  cudaEventRecord(r->ev_pool[i0], r->stream);
  int rc = launch();
  cudaEventRecord(r->ev_pool[i0 + 1], r->stream);
  r->ev_pending.push_back({kind, (int)i0});
  return rc;
}

static int reset_status(eprem_gpu_run *r) {
  DevStatus init{};
  { const double big = DBL_MAX; memcpy(&init.min_tau_bits, &big, sizeof(big)); }
  CK(cudaMemcpyAsync(r->d_status, &init, sizeof(init), cudaMemcpyHostToDevice, r->stream));
  CK(cudaStreamSynchronize(r->stream));
  return EPREM_GPU_OK;
}

static const char *where_name(int w) {
  switch (w) {
    case 1: return "Diffuse Stream Data";
    case 2: return "Adiabatic Focusing";
    case 3: return "Adiabatic Change";
    case 4: return "stream geometry";
    default: return "energetic-particle update";
  }
}

// Reads the status block (synchronising) and reports a device failure.
static int check_status(eprem_gpu_run *r, bool reset_stats, eprem_ep_stats_t *stats) {
  CK(cudaMemcpyAsync(r->h_status, r->d_status, sizeof(DevStatus), cudaMemcpyDeviceToHost,
                     r->stream));
  CK(cudaStreamSynchronize(r->stream));
  const DevStatus st = *r->h_status;
  if (stats) {
    stats->max_subcycles_change = st.max_change;
    stats->max_subcycles_focusing = st.max_focus;
    stats->max_substeps_stream = st.max_stream;
    stats->pad = 0;
    memcpy(&stats->min_tau, &st.min_tau_bits, sizeof(double));
    stats->stream_cell_subcycles = (double)st.stream_cs;
    stats->focus_cell_subcycles = (double)st.focus_cs;
    stats->change_cell_subcycles = (double)st.change_cs;
  }
  if (reset_stats || st.code) {
    int rc = reset_status(r);
    if (rc) return rc;
  }
  if (st.code) {
    char buf[256];
    const char *what = st.code == EPREM_GPU_ERR_NAN       ? "NaN value in"
                       : st.code == EPREM_GPU_ERR_INF     ? "Inf value in"
                       : st.code == EPREM_GPU_ERR_DS      ? "FindSegmentLengths(): Underflow in ds,"
                       : st.code == EPREM_GPU_ERR_SUBCYCLES ? "sub-cycle cap exceeded in"
                       : st.code == EPREM_GPU_ERR_STATE   ? "fewer than 3 nodes left after thinning in"
                                                          : "failure in";
    snprintf(buf, sizeof(buf), "%s %s (stream %d, node %d, energy %d, mu %d)", what,
             where_name(st.where), st.stream, st.node, st.energy, st.mu);
    return fail(st.code, buf);
  }
  return EPREM_GPU_OK;
}

static int validate(const eprem_dims_t *d, const eprem_params_t *p, const eprem_grids_t *g) {
  if (!d || !p || !g) return fail(EPREM_GPU_ERR_ARG, "null argument");
  if (d->num_species != 1)
    return fail(EPREM_GPU_ERR_UNSUPPORTED,
                "num_species must be 1 (the reference indexes egrid by species*E beyond its "
                "length for species > 0)");
  if (d->num_streams < 1 || d->num_streams > 65535) return fail(EPREM_GPU_ERR_ARG, "num_streams out of range");
  if (d->num_nodes < 3) return fail(EPREM_GPU_ERR_ARG, "num_nodes must be >= 3");
  if (d->num_energies < 2 || d->num_energies > 64) return fail(EPREM_GPU_ERR_ARG, "num_energies must be 2..64");
  if (d->num_mu < 2 || d->num_mu > 64) return fail(EPREM_GPU_ERR_ARG, "num_mu must be 2..64");
  if (d->precision != EPREM_FP64 && d->precision != EPREM_FP32) return fail(EPREM_GPU_ERR_ARG, "unknown precision");
  if (p->num_ep_steps < 1) return fail(EPREM_GPU_ERR_ARG, "num_ep_steps must be >= 1");
  if (p->adiabatic_focus_alg < 1 || p->adiabatic_focus_alg > 3 || p->adiabatic_change_alg < 1 ||
      p->adiabatic_change_alg > 3)
    return fail(EPREM_GPU_ERR_ARG, "adiabatic algorithms must be 1, 2 or 3");
  if ((p->adiabatic_focus_alg == 3 && d->num_mu < 4) ||
      (p->adiabatic_change_alg == 3 && d->num_energies < 4))
    return fail(EPREM_GPU_ERR_ARG, "WENO3 needs at least 4 cells along its axis");
  if (p->mfp_type != 1 && p->mfp_type != 2) return fail(EPREM_GPU_ERR_ARG, "mfp_type must be 1 or 2");
  if (!g->egrid || !g->vgrid || !g->vgrid_i || !g->mugrid || !g->rigidity)
    return fail(EPREM_GPU_ERR_ARG, "null grid array");
  return EPREM_GPU_OK;
}

template <typename T>
static cudaError_t dalloc(T **p, size_t n) {
  return cudaMalloc(reinterpret_cast<void **>(p), n * sizeof(T) + 16);
}

extern "C" int eprem_gpu_create(const eprem_dims_t *dims, const eprem_params_t *params,
                                const eprem_grids_t *grids, eprem_gpu_run **out) {
  if (!out) return fail(EPREM_GPU_ERR_ARG, "null output handle");
  *out = nullptr;
  int rc = validate(dims, params, grids);
  if (rc) return rc;
  const int S = dims->num_streams, N = dims->num_nodes, E = dims->num_energies,
            M = dims->num_mu;
  // mu split: cells with mugrid >= 0 take their upwind value from the inner
  // neighbour (src/energeticParticles.c:2379); the grid must be ordered.
  int m0 = M;
  for (int m = 0; m < M; m++)
    if (grids->mugrid[m] >= 0.0) { m0 = m; break; }
  for (int m = 0; m < M; m++)
    if ((grids->mugrid[m] >= 0.0) != (m >= m0))
      return fail(EPREM_GPU_ERR_ARG, "mugrid must be increasing");
  auto *r = new eprem_gpu_run();
  r->dims = *dims;
  r->params = *params;
  r->m0 = m0;
  if (r->params.max_subcycles <= 0) r->params.max_subcycles = 1000000;
  const bool fast32 = dims->precision == EPREM_FP32 && params->adiabatic_focus_alg == 1 &&
                      params->adiabatic_change_alg == 1;
  int prc = plan_stream(dims->precision, N, M, m0, params->stream_variant, &r->splan);
  if (!prc) prc = fast32 ? plan_node32(E, M, &r->nplan) : plan_node(dims->precision, E, M, &r->nplan);
  r->nplan.fast32 = fast32 ? 1 : 0;
  if (prc) {
    delete r;
    return fail(EPREM_GPU_ERR_ARG, "sizes exceed the supported kernel shapes "
                                   "(num_nodes per stream or E*M too large)");
  }
  cudaError_t e = cudaGetDevice(&r->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&r->stream, cudaStreamNonBlocking);
  const size_t SN = r->sn(), cells = r->cells();
  const size_t fbytes = dims->precision == EPREM_FP64 ? sizeof(double) : sizeof(float);
  if (e == cudaSuccess) e = cudaMalloc(&r->d_f, cells * fbytes + 16);
  if (e == cudaSuccess) e = dalloc(&r->d_nodes, (size_t)EPREM_NODE_NFIELDS * SN);
  if (e == cudaSuccess) e = dalloc(&r->d_mugrid, (size_t)M);
  if (e == cudaSuccess) e = dalloc(&r->d_mugrid32, (size_t)M);
  if (e == cudaSuccess && fast32) e = dalloc(&r->d_coef32, SN);
  if (e == cudaSuccess) e = dalloc(&r->d_ec, (size_t)E);
  if (e == cudaSuccess) e = dalloc(&r->d_list, SN);
  if (e == cudaSuccess) e = dalloc(&r->d_list_size, (size_t)S);
  if (e == cudaSuccess) e = dalloc(&r->d_ds_i, SN);
  if (e == cudaSuccess) e = dalloc(&r->d_ds_min, (size_t)S);
  if (e == cudaSuccess) e = dalloc(&r->d_seed_radial, SN);
  if (e == cudaSuccess) e = dalloc(&r->d_mfp_node, SN);
  if (e == cudaSuccess) e = dalloc(&r->d_status, 1);
  if (e == cudaSuccess) e = cudaMallocHost(reinterpret_cast<void **>(&r->h_status), sizeof(DevStatus));
  if (e == cudaSuccess) e = cudaMemsetAsync(r->d_list, 0, SN * sizeof(int), r->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(r->d_list_size, 0, S * sizeof(int), r->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(r->d_nodes, 0, EPREM_NODE_NFIELDS * SN * sizeof(double), r->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(r->d_f, 0, cells * fbytes, r->stream);
  if (e != cudaSuccess) {
    eprem_gpu_destroy(r);
    return cuda_fail(e, "eprem_gpu_create allocation");
  }
  // Per-energy constants with the host libm, as the reference computes them.
  const eprem_params_t &p = r->params;
  std::vector<EnergyConsts> ec(E);
  const double normE1 = 1.0 * kEfac, normE0 = p.bf_ecutoff * kEfac;
  for (int i = 0; i < E; i++) {
    ec[i].egrid = grids->egrid[i];
    ec[i].vgrid = grids->vgrid[i];
    ec[i].vgrid_i = grids->vgrid_i[i];
    ec[i].rig_lamo = grids->rigidity[i] * p.lamo;
    ec[i].seed_power = pow((grids->egrid[i] / normE1), -p.bf_gamma);
    ec[i].seed_exp = exp(-(grids->egrid[i] / normE0));
    ec[i].v32 = (float)grids->vgrid[i];
    ec[i].vi32 = (float)grids->vgrid_i[i];
  }
  std::vector<float> mu32(M);
  for (int m = 0; m < M; m++) mu32[m] = (float)grids->mugrid[m];
  e = cudaMemcpyAsync(r->d_ec, ec.data(), E * sizeof(EnergyConsts), cudaMemcpyHostToDevice, r->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(r->d_mugrid, grids->mugrid, M * sizeof(double), cudaMemcpyHostToDevice, r->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(r->d_mugrid32, mu32.data(), M * sizeof(float), cudaMemcpyHostToDevice, r->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(r->stream);
  if (e != cudaSuccess) {
    eprem_gpu_destroy(r);
    return cuda_fail(e, "eprem_gpu_create upload");
  }
  rc = setup_geometry_attrs(N);
  if (rc) {
    eprem_gpu_destroy(r);
    return fail(rc, "cannot reserve shared memory for the stream-list kernel");
  }
  r->norm_radius = p.bf_r0 / p.r_scale;
  r->neg_beta = -p.bf_beta;
  RunView &v = r->v;
  v.S = S; v.N = N; v.E = E; v.M = M;
  v.precision = dims->precision;
  v.f = r->d_f;
  v.nodes = r->d_nodes;
  v.mugrid = r->d_mugrid;
  v.mugrid32 = r->d_mugrid32;
  v.coef32 = r->d_coef32;
  v.ec = r->d_ec;
  v.list = r->d_list;
  v.list_size = r->d_list_size;
  v.ds_i = r->d_ds_i;
  v.ds_min = r->d_ds_min;
  v.seed_radial = r->d_seed_radial;
  v.mfp_node = r->d_mfp_node;
  v.status = r->d_status;
  v.r_scale = p.r_scale;
  v.dt = p.t_del / (1.0 * p.num_ep_steps);  // src/energeticParticles.c:99
  v.dt_full = v.dt * p.num_ep_steps;        // :861, :1582
  v.dmu = grids->dmu;
  v.dlnp = grids->dlnp;
  v.norm_j0 = p.bf_amplitude * (kMp * kC) / (kMhdDensityNorm * kMev);
  v.bf_xi = p.bf_xi;
  v.dsh_min = p.dsh_min;
  v.damp_cooling = p.damp_cooling;
  v.num_ep_steps = p.num_ep_steps;
  v.max_subcycles = p.max_subcycles;
  v.check_seed = p.check_seed_population > 0;
  v.use_bc = (p.use_ep_boundary > 0) && (p.use_boundary_function > 0);
  v.use_stream = p.use_parallel_diffusion > 0;
  v.use_focus = p.use_adiabatic_focus > 0;
  v.use_change = p.use_adiabatic_change > 0;
  v.relax_in_stream = 1;
  v.focus_alg = p.adiabatic_focus_alg;
  v.change_alg = p.adiabatic_change_alg;
  MhdParams &mh = r->mhd;
  mh.r_scale = p.r_scale; mh.t_del = p.t_del; mh.mhd_us = p.mhd_us; mh.mhd_ns_au = p.mhd_ns_au;
  mh.mhd_bs_au = p.mhd_bs_au; mh.omega_sun = p.omega_sun; mh.ideal_shock = p.ideal_shock;
  mh.sharp = p.ideal_shock_sharpness; mh.scale_len = p.ideal_shock_scale_length;
  mh.jump = p.ideal_shock_jump; mh.falloff = p.ideal_shock_falloff;
  mh.speed = p.ideal_shock_speed; mh.init_time = p.ideal_shock_init_time;
  mh.theta = p.ideal_shock_theta; mh.phi = p.ideal_shock_phi; mh.width = p.ideal_shock_width;
  rc = reset_status(r);
  if (rc) {
    eprem_gpu_destroy(r);
    return rc;
  }
  *out = r;
  g_last_error.clear();
  return EPREM_GPU_OK;
}

extern "C" int eprem_gpu_destroy(eprem_gpu_run *r) {
  if (!r) return EPREM_GPU_OK;
  if (r->stream) cudaStreamSynchronize(r->stream);
  cudaFree(r->d_f);
  cudaFree(r->d_nodes);
  cudaFree(r->d_mugrid);
  cudaFree(r->d_mugrid32);
  cudaFree(r->d_surr_counts);
  cudaFree(r->d_reject);
  cudaFree(r->d_coef32);
  cudaFree(r->d_ec);
  cudaFree(r->d_list);
  cudaFree(r->d_list_size);
  cudaFree(r->d_ds_i);
  cudaFree(r->d_ds_min);
  cudaFree(r->d_seed_radial);
  cudaFree(r->d_mfp_node);
  cudaFree(r->d_status);
  cudaFree(r->d_stage);
  cudaFree(r->d_flux);
  for (cudaEvent_t ev : r->ev_pool) cudaEventDestroy(ev);
  for (auto &slot : r->mas_allocs)
    for (void *p : slot) cudaFree(p);
  if (r->h_status) cudaFreeHost(r->h_status);
  if (r->stream) cudaStreamDestroy(r->stream);
  delete r;
  return EPREM_GPU_OK;
}

static int ensure_stage(eprem_gpu_run *r, size_t elems) {
  if (r->stage_elems >= elems) return EPREM_GPU_OK;
  cudaFree(r->d_stage);
  r->d_stage = nullptr;
  r->stage_elems = 0;
  CK(cudaMalloc(&r->d_stage, elems * sizeof(double)));
  r->stage_elems = elems;
  return EPREM_GPU_OK;
}

// Chunk of doubles staged at a time when converting f for the FP32 form.
static const size_t kStageChunk = (size_t)1 << 27;

extern "C" int eprem_gpu_upload_f(eprem_gpu_run *r, const double *f) {
  if (!r || !f) return fail(EPREM_GPU_ERR_ARG, "null argument");
  const size_t n = r->cells();
  if (r->dims.precision == EPREM_FP64) {
    CK(cudaMemcpyAsync(r->d_f, f, n * sizeof(double), cudaMemcpyHostToDevice, r->stream));
    return EPREM_GPU_OK;
  }
  const size_t chunk = n < kStageChunk ? n : kStageChunk;
  int rc = ensure_stage(r, chunk);
  if (rc) return rc;
  for (size_t off = 0; off < n; off += chunk) {
    const size_t c = (n - off) < chunk ? (n - off) : chunk;
    CK(cudaMemcpyAsync(r->d_stage, f + off, c * sizeof(double), cudaMemcpyHostToDevice, r->stream));
    rc = launch_convert_f(r->v, r->d_stage,
                          reinterpret_cast<double *>(static_cast<float *>(r->d_f) + off), 1, c,
                          r->stream, &r->launches);
    if (rc) return fail(rc, "conversion kernel launch failed");
  }
  return EPREM_GPU_OK;
}

extern "C" int eprem_gpu_download_f(eprem_gpu_run *r, double *f) {
  if (!r || !f) return fail(EPREM_GPU_ERR_ARG, "null argument");
  const size_t n = r->cells();
  if (r->dims.precision == EPREM_FP64) {
    CK(cudaMemcpyAsync(f, r->d_f, n * sizeof(double), cudaMemcpyDeviceToHost, r->stream));
  } else {
    const size_t chunk = n < kStageChunk ? n : kStageChunk;
    int rc = ensure_stage(r, chunk);
    if (rc) return rc;
    for (size_t off = 0; off < n; off += chunk) {
      const size_t c = (n - off) < chunk ? (n - off) : chunk;
      rc = launch_convert_f(r->v,
                            reinterpret_cast<const double *>(static_cast<const float *>(r->d_f) + off),
                            r->d_stage, 0, c, r->stream, &r->launches);
      if (rc) return fail(rc, "conversion kernel launch failed");
      CK(cudaMemcpyAsync(f + off, r->d_stage, c * sizeof(double), cudaMemcpyDeviceToHost, r->stream));
    }
  }
  return check_status(r, false, nullptr);
}

extern "C" int eprem_gpu_upload_nodes(eprem_gpu_run *r, const double *nodes, uint64_t mask) {
  if (!r || !nodes) return fail(EPREM_GPU_ERR_ARG, "null argument");
  const size_t SN = r->sn();
  for (int fld = 0; fld < EPREM_NODE_NFIELDS; fld++)
    if (mask & (1ull << fld))
      CK(cudaMemcpyAsync(r->d_nodes + fld * SN, nodes + fld * SN, SN * sizeof(double),
                         cudaMemcpyHostToDevice, r->stream));
  return EPREM_GPU_OK;
}

extern "C" int eprem_gpu_download_nodes(eprem_gpu_run *r, double *nodes, uint64_t mask) {
  if (!r || !nodes) return fail(EPREM_GPU_ERR_ARG, "null argument");
  const size_t SN = r->sn();
  for (int fld = 0; fld < EPREM_NODE_NFIELDS; fld++)
    if (mask & (1ull << fld))
      CK(cudaMemcpyAsync(nodes + fld * SN, r->d_nodes + fld * SN, SN * sizeof(double),
                         cudaMemcpyDeviceToHost, r->stream));
  return check_status(r, false, nullptr);
}

static int split_node_phase(eprem_gpu_run *r);

extern "C" int eprem_gpu_update_energetic_particles(eprem_gpu_run *r, double t_global) {
  (void)t_global;
  if (!r) return fail(EPREM_GPU_ERR_ARG, "null run");
  const eprem_params_t &p = r->params;
  int rc = timed(r, EPREM_KERNEL_GEOMETRY, [&] {
    return launch_geometry(r->v, r->stream, r->norm_radius, r->neg_beta, p.mfp_type,
                           p.mfp_type == 2 ? p.mfp_b_power : p.mfp_radial_power, p.mhd_bs_au,
                           &r->launches);
  });
  if (rc) return cuda_fail(cudaGetLastError(), "geometry launch");
  if (r->nplan.fast32 && (r->v.use_focus || r->v.use_change)) {
    rc = timed(r, EPREM_KERNEL_NODE,
               [&] { return launch_node32_setup(r->v, r->stream, &r->launches); });
    if (rc) return cuda_fail(cudaGetLastError(), "focusing/change set-up launch");
  }
  for (int step = 0; step < p.num_ep_steps; step++) {
    if (r->v.use_stream)
      rc = timed(r, EPREM_KERNEL_STREAM,
                 [&] { return launch_stream(r->v, r->splan, r->m0, r->stream, &r->launches); });
    else if (r->v.check_seed)
      rc = timed(r, EPREM_KERNEL_SEED_CHECK,
                 [&] { return launch_seed_check(r->v, r->stream, &r->launches); });
    if (rc) return cuda_fail(cudaGetLastError(), "streaming launch");
    if (r->node_mode != EPREM_NODE_PHASE_REFERENCE) {
      rc = timed(r, EPREM_KERNEL_NODE, [&] { return split_node_phase(r); });
      if (rc) return rc == EPREM_GPU_ERR_CUDA ? cuda_fail(cudaGetLastError(), "split node phase") : rc;
    } else if (r->v.use_focus || r->v.use_change) {
      rc = timed(r, EPREM_KERNEL_NODE, [&] {
        return r->nplan.fast32 ? launch_node32(r->v, r->nplan, r->stream, &r->launches)
                               : launch_node(r->v, r->nplan, r->stream, &r->launches);
      });
      if (rc) return cuda_fail(cudaGetLastError(), "focusing/change launch");
    }
  }
  return EPREM_GPU_OK;
}

extern "C" int eprem_gpu_read_stats(eprem_gpu_run *r, eprem_ep_stats_t *stats) {
  if (!r || !stats) return fail(EPREM_GPU_ERR_ARG, "null argument");
  return check_status(r, true, stats);
}

extern "C" int eprem_gpu_update_mhd(eprem_gpu_run *r, double t_global) {
  if (!r) return fail(EPREM_GPU_ERR_ARG, "null run");
  if (r->mas_on) {
    if (!r->mas_selected)
      return fail(EPREM_GPU_ERR_STATE, "MAS background: no time slices selected");
    if (timed(r, EPREM_KERNEL_MHD, [&] {
          return launch_mas_update_mhd(r->v, r->mv, r->params.t_del, r->stream, &r->launches);
        }))
      return cuda_fail(cudaGetLastError(), "updateMhd (MAS) launch");
    return EPREM_GPU_OK;
  }
  if (timed(r, EPREM_KERNEL_MHD,
            [&] { return launch_update_mhd(r->v, r->mhd, t_global, r->stream, &r->launches); }))
    return cuda_fail(cudaGetLastError(), "updateMhd launch");
  return EPREM_GPU_OK;
}

extern "C" int eprem_gpu_mas_init(eprem_gpu_run *r, const eprem_mas_params_t *mp) {
  if (!r || !mp) return fail(EPREM_GPU_ERR_ARG, "null argument");
  if (mp->max_slices < 2 || mp->max_slices > 4096)
    return fail(EPREM_GPU_ERR_ARG, "max_slices must be 2..4096");
  r->mas_ready = true;
  r->mas_on = true;
  r->mas_selected = false;
  r->mas_allocs.assign(mp->max_slices, {});
  r->mas_slots.assign(mp->max_slices, MasSlotDev{});
  r->mas_loaded.assign(mp->max_slices, 0);
  r->mv.radial_max = mp->radial_max;
  r->mv.v_min = mp->v_min;
  r->mv.cor_rotate_fake = mp->cor_rotate_fake;
  r->mv.rotate_solution = mp->rotate_solution;
  r->mv.r_scale = r->params.r_scale;
  r->mv.omega_sun = r->params.omega_sun;
  return EPREM_GPU_OK;
}

extern "C" int eprem_gpu_mas_load_slice(eprem_gpu_run *r, int slot, const eprem_mas_slice_t *s) {
  if (!r || !s) return fail(EPREM_GPU_ERR_ARG, "null argument");
  if (!r->mas_ready) return fail(EPREM_GPU_ERR_STATE, "eprem_gpu_mas_init first");
  if (slot < 0 || slot >= (int)r->mas_slots.size()) return fail(EPREM_GPU_ERR_ARG, "slot out of range");
  CK(cudaStreamSynchronize(r->stream));
  for (void *p : r->mas_allocs[slot]) cudaFree(p);
  r->mas_allocs[slot].clear();
  r->mas_loaded[slot] = 0;
  MasSlotDev dev{};
  for (int f = 0; f < EPREM_MAS_NFIELDS; f++) {
    size_t n = 1;
    for (int a = 0; a < 3; a++) {
      const int d = s->dims[f][a];
      if (d < 2 || !s->mesh[f][a]) return fail(EPREM_GPU_ERR_ARG, "MAS meshes need >= 2 points");
      n *= (size_t)d;
      float *m = nullptr;
      CK(cudaMalloc(&m, d * sizeof(float)));
      r->mas_allocs[slot].push_back(m);
      CK(cudaMemcpy(m, s->mesh[f][a], d * sizeof(float), cudaMemcpyHostToDevice));
      dev.mesh[f][a] = m;
      dev.dims[f][a] = d;
    }
    if (!s->data[f]) return fail(EPREM_GPU_ERR_ARG, "null MAS field");
    float *v = nullptr;
    CK(cudaMalloc(&v, n * sizeof(float)));
    r->mas_allocs[slot].push_back(v);
    CK(cudaMemcpy(v, s->data[f], n * sizeof(float), cudaMemcpyHostToDevice));
    dev.data[f] = v;
  }
  r->mas_slots[slot] = dev;
  r->mas_loaded[slot] = 1;
  return EPREM_GPU_OK;
}

extern "C" int eprem_gpu_mas_select(eprem_gpu_run *r, int slot0, int slot1, double s_cor,
                                    double phi_offset) {
  if (!r) return fail(EPREM_GPU_ERR_ARG, "null run");
  if (!r->mas_ready) return fail(EPREM_GPU_ERR_STATE, "eprem_gpu_mas_init first");
  const int n = (int)r->mas_slots.size();
  if (slot0 < 0 || slot0 >= n || slot1 < 0 || slot1 >= n || !r->mas_loaded[slot0] ||
      !r->mas_loaded[slot1])
    return fail(EPREM_GPU_ERR_ARG, "MAS slot not loaded");
  r->mv.s0 = r->mas_slots[slot0];
  r->mv.s1 = r->mas_slots[slot1];
  r->mv.s_cor = s_cor;
  r->mv.phi_offset = phi_offset;
  r->mas_selected = true;
  return EPREM_GPU_OK;
}

extern "C" int eprem_gpu_mas_use(eprem_gpu_run *r, int use_mas) {
  if (!r) return fail(EPREM_GPU_ERR_ARG, "null run");
  if (!r->mas_ready) return fail(EPREM_GPU_ERR_STATE, "eprem_gpu_mas_init first");
  r->mas_on = use_mas != 0;
  return EPREM_GPU_OK;
}

extern "C" int eprem_gpu_mas_move_nodes(eprem_gpu_run *r, double dt) {
  if (!r) return fail(EPREM_GPU_ERR_ARG, "null run");
  if (!r->mas_ready || !r->mas_selected)
    return fail(EPREM_GPU_ERR_STATE, "MAS background not initialised or no slices selected");
  if (timed(r, EPREM_KERNEL_MOVE,
            [&] { return launch_mas_move_nodes(r->v, r->mv, dt, r->stream, &r->launches); }))
    return cuda_fail(cudaGetLastError(), "masMoveNodes launch");
  return EPREM_GPU_OK;
}

extern "C" int eprem_gpu_move_nodes(eprem_gpu_run *r, double dt) {
  if (!r) return fail(EPREM_GPU_ERR_ARG, "null run");
  if (timed(r, EPREM_KERNEL_MOVE,
            [&] { return launch_move_nodes(r->v, dt, r->stream, &r->launches); }))
    return cuda_fail(cudaGetLastError(), "moveNodes launch");
  return EPREM_GPU_OK;
}

extern "C" int eprem_gpu_omni_flux(eprem_gpu_run *r, double *out) {
  if (!r || !out) return fail(EPREM_GPU_ERR_ARG, "null argument");
  const size_t n = r->sn() * r->dims.num_energies;
  if (!r->d_flux) CK(cudaMalloc(&r->d_flux, n * sizeof(double)));
  if (timed(r, EPREM_KERNEL_FLUX,
            [&] { return launch_omni_flux(r->v, r->d_flux, r->stream, &r->launches); }))
    return cuda_fail(cudaGetLastError(), "flux launch");
  CK(cudaMemcpyAsync(out, r->d_flux, n * sizeof(double), cudaMemcpyDeviceToHost, r->stream));
  return check_status(r, false, nullptr);
}

// Omnidirectional flux staged in a fixed device buffer, for callers that may
// not allocate once their run is set up (a run set sized to fill the GPU's
// memory, a host that budgets device memory at start-up).  The buffer is a
// file-scope device array, created with the module on each device; its
// address is looked up once per device, with that device current, by the
// first call there, so that call should come before any stream capture.
// Every value is written by the flux kernel before it is copied out, so no
// part of the buffer needs zeroing.  All runs on a device share it: calls
// that overlap in time race on it and must be serialised by the caller.
namespace {
constexpr int kFluxStaticDevices = 64;
__device__ __align__(256) double g_flux_static[EPREM_GPU_FLUX_STATIC_MAX];
std::mutex g_flux_static_mutex;
double *g_flux_static_addr[kFluxStaticDevices] = {};

int flux_static_buffer(int device, double **out) {
  if (device < 0 || device >= kFluxStaticDevices)
    return fail(EPREM_GPU_ERR_ARG, "device ordinal beyond the static flux buffer table");
  std::lock_guard<std::mutex> lock(g_flux_static_mutex);
  if (!g_flux_static_addr[device]) {
    int current = -1;
    CK(cudaGetDevice(&current));
    if (current != device) CK(cudaSetDevice(device));
    void *addr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&addr, g_flux_static);
    if (current != device) CK(cudaSetDevice(current));
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(static flux buffer)");
    g_flux_static_addr[device] = static_cast<double *>(addr);
  }
  *out = g_flux_static_addr[device];
  return EPREM_GPU_OK;
}
}  // namespace

extern "C" int eprem_gpu_omni_flux_static(eprem_gpu_run *r, double *out) {
  if (!r || !out) return fail(EPREM_GPU_ERR_ARG, "null argument");
  const size_t n = r->sn() * r->dims.num_energies;
  if (n > (size_t)EPREM_GPU_FLUX_STATIC_MAX)
    return fail(EPREM_GPU_ERR_ARG,
                "eprem_gpu_omni_flux_static: S*N*E = " + std::to_string(n) +
                    " values exceed the static buffer's " +
                    std::to_string(EPREM_GPU_FLUX_STATIC_MAX) + "; use eprem_gpu_omni_flux");
  double *buf = nullptr;
  const int rc = flux_static_buffer(r->device, &buf);
  if (rc) return rc;
  if (launch_omni_flux(r->v, buf, r->stream, &r->launches))
    return cuda_fail(cudaGetLastError(), "flux launch");
  CK(cudaMemcpyAsync(out, buf, n * sizeof(double), cudaMemcpyDeviceToHost, r->stream));
  return check_status(r, false, nullptr);
}

extern "C" int eprem_gpu_synchronize(eprem_gpu_run *r) {
  if (!r) return fail(EPREM_GPU_ERR_ARG, "null run");
  return check_status(r, false, nullptr);
}

extern "C" int eprem_gpu_set_kernel_timing(eprem_gpu_run *r, int enable) {
  if (!r) return fail(EPREM_GPU_ERR_ARG, "null run");
  CK(cudaStreamSynchronize(r->stream));
  r->timing = enable != 0;
  r->ev_pending.clear();
  r->ev_used = 0;
  return EPREM_GPU_OK;
}

extern "C" int eprem_gpu_read_kernel_timing(eprem_gpu_run *r, eprem_kernel_time_t *out) {
  if (!r || !out) return fail(EPREM_GPU_ERR_ARG, "null argument");
  CK(cudaStreamSynchronize(r->stream));
  for (int k = 0; k < EPREM_KERNEL_NKINDS; k++) out[k] = eprem_kernel_time_t{0, 0, 0.0};
  for (const auto &pe : r->ev_pending) {
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, r->ev_pool[pe.second], r->ev_pool[pe.second + 1]));
    out[pe.first].launches += 1;
    out[pe.first].total_ms += ms;
  }
  r->ev_pending.clear();
  r->ev_used = 0;
  return EPREM_GPU_OK;
}

extern "C" void *eprem_gpu_stream(eprem_gpu_run *r) { return r ? (void *)r->stream : nullptr; }

extern "C" uint64_t eprem_gpu_kernel_launches(const eprem_gpu_run *r) {
  return r ? r->launches : 0;
}

extern "C" const char *eprem_gpu_last_error(void) { return g_last_error.c_str(); }

extern "C" int eprem_gpu_init_seed_population(eprem_gpu_run *r, uint64_t seed,
                                              double perturbation) {
  if (!r) return fail(EPREM_GPU_ERR_ARG, "null run");
  const eprem_params_t &p = r->params;
  if (launch_geometry(r->v, r->stream, r->norm_radius, r->neg_beta, p.mfp_type,
                      p.mfp_type == 2 ? p.mfp_b_power : p.mfp_radial_power, p.mhd_bs_au,
                      &r->launches) ||
      launch_seed_population(r->v, (unsigned long long)seed, perturbation, r->stream,
                             &r->launches))
    return cuda_fail(cudaGetLastError(), "seed population launch");
  return check_status(r, false, nullptr);
}

// ---- autotuner ---------------------------------------------------------------
// Times the FP32 streaming-kernel shapes on a scratch copy of the run's first
// streams (the kernel that takes 90 % of a step) and keeps the fastest.  The
// copy has its own status block, so the run's statistics are untouched.
namespace {
constexpr int kTuneVariants[] = {5, 4, 3, 2, 1};

int tune_stream(eprem_gpu_run *r, int *chosen) {
  const eprem_params_t &p = r->params;
  CK(cudaStreamSynchronize(r->stream));
  int rc = launch_geometry(r->v, r->stream, r->norm_radius, r->neg_beta, p.mfp_type,
                           p.mfp_type == 2 ? p.mfp_b_power : p.mfp_radial_power, p.mhd_bs_au,
                           &r->launches);
  if (rc) return cuda_fail(cudaGetLastError(), "autotune geometry launch");
  const int S_sub = r->dims.num_streams < 96 ? r->dims.num_streams : 96;
  const size_t n = (size_t)S_sub * r->dims.num_nodes * r->dims.num_energies * r->dims.num_mu;
  void *f = nullptr;
  DevStatus *st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaMalloc(&f, n * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&st, sizeof(DevStatus));
  if (e == cudaSuccess) e = cudaMemsetAsync(st, 0, sizeof(DevStatus), r->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(f, r->d_f, n * sizeof(float), cudaMemcpyDeviceToDevice, r->stream);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  RunView v = r->v;
  v.S = S_sub;
  v.f = f;
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
// updateEnergeticParticles, t += tDel) into one CUDA graph, each run on its
// own branch between a fork and a join on the ensemble's stream; every step
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
  for (int i = 0; i < n && err == cudaSuccess && rc == EPREM_GPU_OK; i++) {
    eprem_gpu_run *r = e->runs[i];
    r->timing = false;  // no event bookkeeping inside a graph
    const uint64_t l0 = r->launches;
    err = cudaStreamWaitEvent(r->stream, e->fork, 0);
    if (err != cudaSuccess) break;
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
    if (err == cudaSuccess) err = cudaStreamWaitEvent(e->origin, e->joins[i], 0);
  }
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

extern "C" int eprem_gpu_ensemble_step(eprem_gpu_ensemble *e) {
  if (!e) return fail(EPREM_GPU_ERR_ARG, "null ensemble");
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

// ---- surrogate building blocks ---------------------------------------------
namespace {
std::mutex g_gemm_err_mutex;
int *g_gemm_err[kFluxStaticDevices] = {};
}  // namespace

extern "C" int eprem_gpu_gemm_bf16(const void *A, int lda, const void *Bt, int ldb,
                                   const float *bias, float *C, int ldc, int M, int N, int K,
                                   void *stream) {
  if (!A || !Bt || !C) return fail(EPREM_GPU_ERR_ARG, "null operand");
  int dev = 0;
  CK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kFluxStaticDevices) return fail(EPREM_GPU_ERR_ARG, "device ordinal");
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

extern "C" int eprem_gpu_surrogate_set_tolerance(eprem_gpu_surrogate *s, double tol) {
  if (!s) return fail(EPREM_GPU_ERR_ARG, "null surrogate");
  s->tol = (float)tol;
  return EPREM_GPU_OK;
}

// Node phase of the split and surrogate forms, one EP sub-step.
static int split_node_phase(eprem_gpu_run *r) {
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
