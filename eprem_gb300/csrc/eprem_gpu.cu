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

#include "run.h"

using namespace eprem;

namespace eprem {
namespace {
thread_local std::string g_last_error;
const double kEfac = kMev / (kMp * kC * kC);
}  // namespace

int fail(int code, const std::string &msg) {
  g_last_error = msg;
  return code;
}

int cuda_fail(cudaError_t e, const char *what) {
  return fail(EPREM_GPU_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
}  // namespace eprem

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
    case 6: return "DiffuseShellData";
    default: return "energetic-particle update";
  }
}

// Reads the status block (synchronising) and reports a device failure.
int eprem::check_status(eprem_gpu_run *r, bool reset_stats, eprem_ep_stats_t *stats) {
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

namespace {
int flux_static_buffer(int device, double **out);
}
static int mas_mark_used(eprem_gpu_run *r);

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
  const bool bc = params->use_ep_boundary > 0 && params->use_boundary_function > 0;
  int prc = plan_stream(dims->precision, N, M, m0, params->stream_variant, bc, &r->splan);
  if (!prc) prc = fast32 ? plan_node32(E, M, &r->nplan) : plan_node(dims->precision, E, M, &r->nplan);
  r->nplan.fast32 = fast32 ? 1 : 0;
  if (prc) {
    delete r;
    return fail(EPREM_GPU_ERR_ARG, "sizes exceed the supported kernel shapes "
                                   "(num_nodes per stream or E*M too large)");
  }
  cudaError_t e = cudaGetDevice(&r->device);
  // the static flux buffer's module is loaded (and its 8 MiB made resident)
  // here, before this run's own allocations, so that a run set sized to fill
  // the device never meets that load later
  double *flux_static = nullptr;
  if (e == cudaSuccess && flux_static_buffer(r->device, &flux_static) != EPREM_GPU_OK) {
    delete r;
    return EPREM_GPU_ERR_CUDA;  // the message is set
  }
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&r->stream, cudaStreamNonBlocking);
  const size_t SN = r->sn(), cells = r->cells();
  const size_t fbytes = dims->precision == EPREM_FP64 ? sizeof(double) : sizeof(float);
  if (e == cudaSuccess) e = cudaMalloc(&r->d_f, cells * fbytes + 16);
  if (e == cudaSuccess && dims->precision == EPREM_FP32) e = dalloc(&r->d_fexp, SN * E);
  if (e == cudaSuccess && r->d_fexp)
    e = cudaMemsetAsync(r->d_fexp, 0, SN * E * sizeof(short), r->stream);
  if (e == cudaSuccess) e = dalloc(&r->d_nodes, (size_t)EPREM_NODE_NFIELDS * SN);
  if (e == cudaSuccess) e = dalloc(&r->d_mugrid, (size_t)M);
  if (e == cudaSuccess) e = dalloc(&r->d_mugrid32, (size_t)M);
  if (e == cudaSuccess && fast32) e = dalloc(&r->d_coef32, SN);
  // FP32 streaming coefficients (any FP32 run may be tuned to stream2.cu)
  if (e == cudaSuccess && dims->precision == EPREM_FP32 && params->use_parallel_diffusion > 0)
    e = dalloc(&r->d_scoef, SN * (size_t)dims->num_energies);
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
  const double norm_j0 = p.bf_amplitude * (kMp * kC) / (kMhdDensityNorm * kMev);
  for (int i = 0; i < E; i++) {
    ec[i].egrid = grids->egrid[i];
    ec[i].vgrid = grids->vgrid[i];
    ec[i].vgrid_i = grids->vgrid_i[i];
    ec[i].rig_lamo = grids->rigidity[i] * p.lamo;
    ec[i].seed_power = pow((grids->egrid[i] / normE1), -p.bf_gamma);
    ec[i].seed_exp = exp(-(grids->egrid[i] / normE0));
    ec[i].v32 = (float)grids->vgrid[i];
    ec[i].vi32 = (float)grids->vgrid_i[i];
    ec[i].dvi32 = (i >= 1 && i + 1 < E)
                      ? (float)(grids->vgrid_i[i + 1] - grids->vgrid_i[i - 1]) : 0.f;
    // the energy-only factor of sepSeedFunction, normalised to [1, 2) by 2^seed_k
    const double ce = norm_j0 * ec[i].seed_power * ec[i].seed_exp / p.bf_xi / (2.0 * ec[i].egrid);
    ec[i].seed_k = (std::isfinite(ce) && ce >= DBL_MIN) ? -ilogb(ce) : 1022;
  }
  std::vector<float> mu32(M);
  for (int m = 0; m < M; m++) mu32[m] = (float)grids->mugrid[m];
  for (int i = 0; i < E; i++) ec[i].drift_factor = 0.0;
  r->h_ec = ec;
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
  r->grid_dlnp = grids->dlnp;
  r->norm_radius = p.bf_r0 / p.r_scale;
  r->neg_beta = -p.bf_beta;
  RunView &v = r->v;
  v.S = S; v.N = N; v.E = E; v.M = M;
  v.precision = dims->precision;
  v.f = r->d_f;
  v.fexp = r->d_fexp;
  v.nodes = r->d_nodes;
  v.mugrid = r->d_mugrid;
  v.mugrid32 = r->d_mugrid32;
  v.coef32 = r->d_coef32;
  v.scoef = r->d_scoef;
  v.ec = r->d_ec;
  v.list = r->d_list;
  v.list_size = r->d_list_size;
  v.ds_i = r->d_ds_i;
  v.ds_min = r->d_ds_min;
  v.seed_radial = r->d_seed_radial;
  v.mfp_node = r->d_mfp_node;
  v.status = r->d_status;
  v.node_stride = (size_t)S * N;
  v.s_base = 0;
  v.r_scale = p.r_scale;
  v.dt = p.t_del / (1.0 * p.num_ep_steps);  // src/energeticParticles.c:99
  v.dt_full = v.dt * p.num_ep_steps;        // :861, :1582
  v.dmu = grids->dmu;
  v.dlnp = grids->dlnp;
  v.norm_j0 = norm_j0;
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
  if (r->copy_stream) cudaStreamSynchronize(r->copy_stream);  // slice copies may be queued
  cudaFree(r->d_f);
  cudaFree(r->d_fexp);
  cudaFree(r->d_shell_fexp);
  cudaFree(r->d_nodes);
  cudaFree(r->d_mugrid);
  cudaFree(r->d_mugrid32);
  cudaFree(r->d_surr_counts);
  cudaFree(r->d_reject);
  cudaFree(r->d_coef32);
  cudaFree(r->d_scoef);
  cudaFree(r->d_ec);
  cudaFree(r->d_list);
  cudaFree(r->d_list_size);
  cudaFree(r->d_ds_i);
  cudaFree(r->d_ds_min);
  cudaFree(r->d_seed_radial);
  cudaFree(r->d_mfp_node);
  cudaFree(r->d_status);
  cudaFree(r->d_stage);
  for (cudaEvent_t ev : r->stage_ev)
    if (ev) cudaEventDestroy(ev);
  if (r->copy_stream) cudaStreamDestroy(r->copy_stream);
  cudaFree(r->d_flux);
  cudaFree(r->d_tmpl);
  cudaFree(r->d_news);
  cudaFree(r->d_shell_ent);
  cudaFree(r->d_shell_del);
  cudaFree(r->d_shell_f);
  cudaFree(r->d_curl);
  cudaFree(r->d_drift_news);
  cudaFree(r->d_drift_ent);
  cudaFree(r->d_drift_del);
  for (cudaEvent_t ev : r->ev_pool) cudaEventDestroy(ev);
  for (auto &slot : r->mas_allocs)
    for (void *p : slot) cudaFree(p);
  for (cudaEvent_t ev : r->mas_ready_ev)
    if (ev) cudaEventDestroy(ev);
  for (cudaEvent_t ev : r->mas_used_ev)
    if (ev) cudaEventDestroy(ev);
  if (r->h_status) cudaFreeHost(r->h_status);
  if (r->stream) cudaStreamDestroy(r->stream);
  delete r;
  return EPREM_GPU_OK;
}

static int ensure_stage(eprem_gpu_run *r, size_t elems) {
  if (!r->copy_stream) {
    CK(cudaStreamCreateWithFlags(&r->copy_stream, cudaStreamNonBlocking));
    for (cudaEvent_t &ev : r->stage_ev) CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  }
  if (r->stage_elems >= elems) return EPREM_GPU_OK;
  cudaFree(r->d_stage);
  r->d_stage = nullptr;
  r->stage_elems = 0;
  CK(cudaMalloc(&r->d_stage, 2 * elems * sizeof(double)));
  r->stage_elems = elems;
  return EPREM_GPU_OK;
}

// Chunk of doubles staged at a time when converting f for the FP32 form:
// whole rows of M cells (each row is converted with its exponent).
static const size_t kStageChunk = (size_t)1 << 27;
static size_t stage_chunk(size_t M) { return kStageChunk / M * M; }

// Upload of an FP32-form f: chunks of FP64 host values through a staging
// buffer, converted on the run's stream (the host-to-device copies run at the
// link's rate in stream order; the conversion is short beside them).
extern "C" int eprem_gpu_upload_f(eprem_gpu_run *r, const double *f) {
  if (!r || !f) return fail(EPREM_GPU_ERR_ARG, "null argument");
  const size_t n = r->cells();
  if (r->dims.precision == EPREM_FP64) {
    CK(cudaMemcpyAsync(r->d_f, f, n * sizeof(double), cudaMemcpyHostToDevice, r->stream));
    return EPREM_GPU_OK;
  }
  const size_t M = r->dims.num_mu;
  const size_t chunk = n < stage_chunk(M) ? n : stage_chunk(M);  // whole rows
  int rc = ensure_stage(r, chunk);
  if (rc) return rc;
  // the copy stream's downloads may still read the staging buffers
  CK(cudaEventRecord(r->stage_ev[2], r->copy_stream));
  CK(cudaStreamWaitEvent(r->stream, r->stage_ev[2], 0));
  size_t k = 0;
  for (size_t off = 0; off < n; off += chunk, ++k) {
    const size_t c = (n - off) < chunk ? (n - off) : chunk;
    double *buf = r->d_stage + (k & 1) * r->stage_elems;
    CK(cudaMemcpyAsync(buf, f + off, c * sizeof(double), cudaMemcpyHostToDevice, r->stream));
    rc = launch_convert_f(r->v, off / M, c / M, buf, 1, r->stream, &r->launches);
    if (rc) return fail(rc, "conversion kernel launch failed");
  }
  return EPREM_GPU_OK;
}

// Download of an FP32-form f: chunk k is converted into staging buffer k%2
// on the run's stream, then copied to the host on the copy stream; the run's
// stream waits for the last copy.
extern "C" int eprem_gpu_download_f(eprem_gpu_run *r, double *f) {
  if (!r || !f) return fail(EPREM_GPU_ERR_ARG, "null argument");
  const size_t n = r->cells();
  if (r->dims.precision == EPREM_FP64) {
    CK(cudaMemcpyAsync(f, r->d_f, n * sizeof(double), cudaMemcpyDeviceToHost, r->stream));
  } else {
    const size_t M = r->dims.num_mu;
    const size_t chunk = n < stage_chunk(M) ? n : stage_chunk(M);  // whole rows
    int rc = ensure_stage(r, chunk);
    if (rc) return rc;
    cudaEvent_t *converted = r->stage_ev, *copied = r->stage_ev + 2;
    CK(cudaEventRecord(copied[0], r->copy_stream));
    CK(cudaEventRecord(copied[1], r->copy_stream));
    size_t k = 0;
    for (size_t off = 0; off < n; off += chunk, ++k) {
      const size_t c = (n - off) < chunk ? (n - off) : chunk;
      double *buf = r->d_stage + (k & 1) * r->stage_elems;
      CK(cudaStreamWaitEvent(r->stream, copied[k & 1], 0));
      rc = launch_convert_f(r->v, off / M, c / M, buf, 0, r->stream, &r->launches);
      if (rc) return fail(rc, "conversion kernel launch failed");
      CK(cudaEventRecord(converted[k & 1], r->stream));
      CK(cudaStreamWaitEvent(r->copy_stream, converted[k & 1], 0));
      CK(cudaMemcpyAsync(f + off, buf, c * sizeof(double), cudaMemcpyDeviceToHost, r->copy_stream));
      CK(cudaEventRecord(copied[k & 1], r->copy_stream));
    }
    CK(cudaEventRecord(copied[0], r->copy_stream));
    CK(cudaStreamWaitEvent(r->stream, copied[0], 0));
  }
  return check_status(r, false, nullptr);
}

static RunView stream_range_view(const eprem_gpu_run *r, int s0, int s1);

// Pitched forms: stream s's N*E*M values at f + s * stream_pitch.  The FP32
// form goes through the staging buffer a group of whole streams at a time.
static int copy_f_pitched(eprem_gpu_run *r, double *host, size_t stream_pitch, bool up) {
  const size_t per = (size_t)r->dims.num_nodes * r->dims.num_energies * r->dims.num_mu;
  const size_t pitch = stream_pitch ? stream_pitch : per;
  if (pitch < per) return fail(EPREM_GPU_ERR_ARG, "stream_pitch below N*E*M");
  if (pitch == per) return up ? eprem_gpu_upload_f(r, host) : eprem_gpu_download_f(r, host);
  const int S = r->dims.num_streams;
  const size_t row = per * sizeof(double);
  if (r->dims.precision == EPREM_FP64) {
    if (up)
      CK(cudaMemcpy2DAsync(r->d_f, row, host, pitch * sizeof(double), row, S,
                           cudaMemcpyHostToDevice, r->stream));
    else
      CK(cudaMemcpy2DAsync(host, pitch * sizeof(double), r->d_f, row, row, S,
                           cudaMemcpyDeviceToHost, r->stream));
    return up ? EPREM_GPU_OK : check_status(r, false, nullptr);
  }
  const int group = std::max(1, (int)std::min<size_t>((size_t)S, kStageChunk / per));
  int rc = ensure_stage(r, (size_t)group * per);
  if (rc) return rc;
  // the copy stream's downloads may still read the staging buffers
  CK(cudaEventRecord(r->stage_ev[2], r->copy_stream));
  CK(cudaStreamWaitEvent(r->stream, r->stage_ev[2], 0));
  for (int s0 = 0; s0 < S; s0 += group) {
    const int ns = std::min(group, S - s0);
    const RunView v = stream_range_view(r, s0, s0 + ns);
    double *buf = r->d_stage;
    const size_t nrows = (size_t)ns * per / r->dims.num_mu;
    if (up) {
      CK(cudaMemcpy2DAsync(buf, row, host + (size_t)s0 * pitch, pitch * sizeof(double), row, ns,
                           cudaMemcpyHostToDevice, r->stream));
      rc = launch_convert_f(v, 0, nrows, buf, 1, r->stream, &r->launches);
    } else {
      rc = launch_convert_f(v, 0, nrows, buf, 0, r->stream, &r->launches);
      if (!rc)
        CK(cudaMemcpy2DAsync(host + (size_t)s0 * pitch, pitch * sizeof(double), buf, row, row, ns,
                             cudaMemcpyDeviceToHost, r->stream));
    }
    if (rc) return fail(rc, "conversion kernel launch failed");
  }
  return up ? EPREM_GPU_OK : check_status(r, false, nullptr);
}

extern "C" int eprem_gpu_upload_f_pitched(eprem_gpu_run *r, const double *f, size_t stream_pitch) {
  if (!r || !f) return fail(EPREM_GPU_ERR_ARG, "null argument");
  return copy_f_pitched(r, const_cast<double *>(f), stream_pitch, true);
}

extern "C" int eprem_gpu_download_f_pitched(eprem_gpu_run *r, double *f, size_t stream_pitch) {
  if (!r || !f) return fail(EPREM_GPU_ERR_ARG, "null argument");
  return copy_f_pitched(r, f, stream_pitch, false);
}

extern "C" int eprem_gpu_ripple_f(eprem_gpu_run *r, const double *tmpl, size_t stream_pitch) {
  if (!r || !tmpl) return fail(EPREM_GPU_ERR_ARG, "null argument");
  const size_t em = (size_t)r->dims.num_energies * r->dims.num_mu;
  const size_t pitch = stream_pitch ? stream_pitch : em;
  if (pitch < em) return fail(EPREM_GPU_ERR_ARG, "stream_pitch below E*M");
  const int S = r->dims.num_streams;
  if (!r->d_tmpl) CK(cudaMalloc(&r->d_tmpl, (size_t)S * em * sizeof(double)));
  CK(cudaMemcpy2DAsync(r->d_tmpl, em * sizeof(double), tmpl, pitch * sizeof(double),
                       em * sizeof(double), S, cudaMemcpyHostToDevice, r->stream));
  if (launch_ripple_f(r->v, r->d_tmpl, r->stream, &r->launches))
    return cuda_fail(cudaGetLastError(), "ripple launch");
  return EPREM_GPU_OK;
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

// The run's view restricted to streams [s0, s1): every per-stream and
// per-node array starts at stream s0; node fields keep the run's stride and
// errors report the run's stream numbers.  Streams are independent on this
// path (no drift, no shell diffusion), so updating the views of a partition
// of the streams one after another is the update of the whole run.
static RunView stream_range_view(const eprem_gpu_run *r, int s0, int s1) {
  const RunView &v = r->v;
  RunView u = v;
  const size_t n0 = (size_t)s0 * v.N;
  const size_t c0 = n0 * v.E * v.M;
  u.S = s1 - s0;
  u.s_base = v.s_base + s0;
  u.f = v.precision == EPREM_FP32 ? static_cast<void *>(static_cast<float *>(v.f) + c0)
                                  : static_cast<void *>(static_cast<double *>(v.f) + c0);
  if (u.fexp) u.fexp = v.fexp + n0 * v.E;
  u.nodes = v.nodes + n0;
  u.list = v.list + n0;
  u.list_size = v.list_size + s0;
  u.ds_i = v.ds_i + n0;
  u.ds_min = v.ds_min + s0;
  u.seed_radial = v.seed_radial + n0;
  u.mfp_node = v.mfp_node + n0;
  if (u.coef32) u.coef32 = v.coef32 + n0;
  if (u.scoef) u.scoef = v.scoef + (size_t)s0 * v.E * v.N;
  return u;
}

// updateEnergeticParticles on the streams of view v, on the run's stream, in
// three pieces (ensembles interleave the sub-steps of several runs):
// ep_begin once per call, then per EP sub-step ep_stream_phase and
// ep_node_phase.
int eprem::ep_begin(eprem_gpu_run *r, const RunView &v) {
  const eprem_params_t &p = r->params;
  int rc = timed(r, EPREM_KERNEL_GEOMETRY, [&] {
    return launch_geometry(v, r->stream, r->norm_radius, r->neg_beta, p.mfp_type,
                           p.mfp_type == 2 ? p.mfp_b_power : p.mfp_radial_power, p.mhd_bs_au,
                           &r->launches);
  });
  if (rc) return cuda_fail(cudaGetLastError(), "geometry launch");
  if (v.use_stream && r->splan.reg_coef == 2) {
    rc = timed(r, EPREM_KERNEL_GEOMETRY,
               [&] { return launch_stream2_coef(v, r->stream, &r->launches); });
    if (rc) return cuda_fail(cudaGetLastError(), "streaming coefficient launch");
  }
  if (r->nplan.fast32 && (v.use_focus || v.use_change)) {
    rc = timed(r, EPREM_KERNEL_NODE,
               [&] { return launch_node32_setup(v, r->stream, &r->launches); });
    if (rc) return cuda_fail(cudaGetLastError(), "focusing/change set-up launch");
  }
  // shell diffusion and drift couple the streams: only a whole-run view
  // reaches here with them on (the stream-range entries route around them)
  if (r->shell_on && &v != &r->v)
    return fail(EPREM_GPU_ERR_UNSUPPORTED, "shell diffusion on a stream range");
  if (r->drift_on && &v != &r->v) return fail(EPREM_GPU_ERR_UNSUPPORTED, "drift on a stream range");
  if (r->shell_on) {
    rc = timed(r, EPREM_KERNEL_SHELL, [&] {
      return launch_shell_coef(v, r->d_news, r->kperxkpar, r->d_shell_del, r->stream,
                               &r->launches);
    });
    if (rc) return cuda_fail(cudaGetLastError(), "shell diffusion set-up launch");
  }
  if (r->drift_on && r->drift_links) {
    rc = timed(r, EPREM_KERNEL_SHELL, [&] {
      return launch_drift_coef(v, r->d_drift_news, r->d_drift_del, r->stream, &r->launches);
    });
    if (rc) return cuda_fail(cudaGetLastError(), "drift set-up launch");
  }
  return EPREM_GPU_OK;
}

int eprem::ep_stream_phase(eprem_gpu_run *r, const RunView &v) {
  int rc = EPREM_GPU_OK;
  if (v.use_stream)
    rc = timed(r, EPREM_KERNEL_STREAM,
               [&] { return launch_stream(v, r->splan, r->m0, r->stream, &r->launches); });
  else if (v.check_seed)
    rc = timed(r, EPREM_KERNEL_SEED_CHECK,
               [&] { return launch_seed_check(v, r->stream, &r->launches); });
  return rc ? cuda_fail(cudaGetLastError(), "streaming launch") : EPREM_GPU_OK;
}

int eprem::ep_node_phase(eprem_gpu_run *r, const RunView &v) {
  int rc = EPREM_GPU_OK;
  if (r->node_mode != EPREM_NODE_PHASE_REFERENCE) {
    rc = timed(r, EPREM_KERNEL_NODE, [&] { return split_node_phase(r); });
    if (rc) return rc == EPREM_GPU_ERR_CUDA ? cuda_fail(cudaGetLastError(), "split node phase") : rc;
  } else if (v.use_focus || v.use_change) {
    rc = timed(r, EPREM_KERNEL_NODE, [&] {
      return r->nplan.fast32 ? launch_node32(v, r->nplan, r->stream, &r->launches)
                             : launch_node(v, r->nplan, r->stream, &r->launches);
    });
    if (rc) return cuda_fail(cudaGetLastError(), "focusing/change launch");
  }
  // (each perpendicular step swaps the run's two f buffers, which v, the
  // run's own view, sees)
  // DiffuseShellData after every stream's sub-step (src/energeticParticles.c:178-182)
  if (r->shell_on) {
    rc = timed(r, EPREM_KERNEL_SHELL, [&] {
      return launch_shell_diffuse(v, r->d_shell_ent, r->shell_L, r->d_shell_del, r->d_shell_f,
                                  r->d_shell_fexp, r->stream, &r->launches);
    });
    if (rc) return cuda_fail(cudaGetLastError(), "shell diffusion launch");
    std::swap(r->d_f, r->d_shell_f);  // the new f is the other buffer
    std::swap(r->d_fexp, r->d_shell_fexp);
    r->v.f = r->d_f;
    r->v.fexp = r->d_fexp;
  }
  // DriftShellData after the shell diffusion (src/energeticParticles.c:186-190)
  if (r->drift_on && r->drift_links) {
    rc = timed(r, EPREM_KERNEL_SHELL, [&] {
      return launch_shell_diffuse(v, r->d_drift_ent, r->drift_L, r->d_drift_del, r->d_shell_f,
                                  r->d_shell_fexp, r->stream, &r->launches, true);
    });
    if (rc) return cuda_fail(cudaGetLastError(), "drift launch");
    std::swap(r->d_f, r->d_shell_f);
    std::swap(r->d_fexp, r->d_shell_fexp);
    r->v.f = r->d_f;
    r->v.fexp = r->d_fexp;
  }
  return EPREM_GPU_OK;
}

static int ep_update(eprem_gpu_run *r, const RunView &v) {
  int rc = ep_begin(r, v);
  for (int step = 0; step < r->params.num_ep_steps && !rc; step++) {
    rc = ep_stream_phase(r, v);
    if (!rc) rc = ep_node_phase(r, v);
  }
  return rc;
}

extern "C" int eprem_gpu_update_energetic_particles(eprem_gpu_run *r, double t_global) {
  (void)t_global;
  if (!r) return fail(EPREM_GPU_ERR_ARG, "null run");
  return ep_update(r, r->v);
}

// The same update with f in host memory, pipelined: the streams go through in
// chunks; chunk c's host-to-device copy runs on the copy stream while chunk
// c-1 is updated on the run's stream, and its device-to-host copy while chunk
// c+1 is updated (measured on a GB300 whose host link moved 31 GB/s back:
// 0.26-0.30 s of copies left per 4.81 s step with eight equal chunks).  The FP32 form converts each chunk in one of two staging
// buffers (chunk c in buffer c % 2, reused once chunk c-2's copy back has
// left it).  Synchronous: f_out holds the result on return.
extern "C" int eprem_gpu_update_energetic_particles_host(eprem_gpu_run *r, const double *f_in,
                                                         double *f_out, size_t stream_pitch,
                                                         double t_global) {
  (void)t_global;
  if (!r || !f_in || !f_out) return fail(EPREM_GPU_ERR_ARG, "null argument");
  const int S = r->dims.num_streams;
  const size_t per_stream = (size_t)r->dims.num_nodes * r->dims.num_energies * r->dims.num_mu;
  const size_t pitch = stream_pitch ? stream_pitch : per_stream;
  if (pitch < per_stream) return fail(EPREM_GPU_ERR_ARG, "stream_pitch below N*E*M");
  if (r->node_mode != EPREM_NODE_PHASE_REFERENCE || r->shell_on || r->drift_on) {
    // those phases, shell diffusion and drift work on the whole run
    int rc = eprem_gpu_upload_f_pitched(r, f_in, pitch);
    if (!rc) rc = ep_update(r, r->v);
    if (!rc) rc = eprem_gpu_download_f_pitched(r, f_out, pitch);
    return rc;
  }
  // Chunks: a short first and last one (1/32 of the streams each: the first
  // upload and the last download are the copies nothing hides) around six
  // long ones, whose copies each take less than a neighbour's update.
  std::vector<int> bounds{0};
  const int edge = S >= 64 ? (S + 31) / 32 : (S >= 8 ? 1 : 0);
  if (edge) {
    const int mid = S - 2 * edge;
    bounds.push_back(edge);
    for (int i = 1; i <= 6; i++) {
      const int b = edge + (int)((long long)mid * i / 6);
      if (b > bounds.back()) bounds.push_back(b);
    }
  }
  if (bounds.back() < S) bounds.push_back(S);
  const int nch = (int)bounds.size() - 1;
  int widest = 0;
  for (int c = 0; c < nch; c++) widest = std::max(widest, bounds[c + 1] - bounds[c]);
  const bool fp32 = r->dims.precision == EPREM_FP32;
  int rc = ensure_stage(r, fp32 ? (size_t)widest * per_stream : 1);
  if (rc) return rc;
  cudaEvent_t *arrived = r->stage_ev, *updated = r->stage_ev + 2;
  // the run's earlier work on f and the staging buffers comes first
  CK(cudaEventRecord(updated[0], r->stream));
  CK(cudaStreamWaitEvent(r->copy_stream, updated[0], 0));
  auto dev64 = [&](int c) {  // chunk c on the device as FP64: staging or f itself
    return fp32 ? r->d_stage + (size_t)(c & 1) * r->stage_elems
                : static_cast<double *>(r->d_f) + (size_t)bounds[c] * per_stream;
  };
  const size_t row = per_stream * sizeof(double);
  auto h2d = [&](int c) -> int {
    const size_t rows = (size_t)(bounds[c + 1] - bounds[c]);
    if (pitch == per_stream)
      CK(cudaMemcpyAsync(dev64(c), f_in + (size_t)bounds[c] * pitch, rows * row,
                         cudaMemcpyHostToDevice, r->copy_stream));
    else
      CK(cudaMemcpy2DAsync(dev64(c), row, f_in + (size_t)bounds[c] * pitch,
                           pitch * sizeof(double), row, rows, cudaMemcpyHostToDevice,
                           r->copy_stream));
    CK(cudaEventRecord(arrived[c & 1], r->copy_stream));
    return EPREM_GPU_OK;
  };
  // Per chunk, the update is queued first, then the next chunk's upload and
  // this chunk's download: the device has the update to run even while the
  // host sits in a copy call.
  rc = h2d(0);
  for (int c = 0; c < nch && !rc; c++) {
    const int s0 = bounds[c], s1 = bounds[c + 1];
    const size_t n = (size_t)(s1 - s0) * per_stream;
    const RunView v = stream_range_view(r, s0, s1);
    CK(cudaStreamWaitEvent(r->stream, arrived[c & 1], 0));
    if (fp32) {
      rc = launch_convert_f(v, 0, n / r->dims.num_mu, dev64(c), 1, r->stream, &r->launches);
      if (rc) return fail(rc, "conversion kernel launch failed");
    }
    rc = ep_update(r, v);
    if (rc) break;
    if (fp32) {
      rc = launch_convert_f(v, 0, n / r->dims.num_mu, dev64(c), 0, r->stream, &r->launches);
      if (rc) return fail(rc, "conversion kernel launch failed");
    }
    CK(cudaEventRecord(updated[c & 1], r->stream));
    if (c + 1 < nch) rc = h2d(c + 1);  // copy stream: after chunk c-1's download
    if (rc) break;
    CK(cudaStreamWaitEvent(r->copy_stream, updated[c & 1], 0));
    if (pitch == per_stream)
      CK(cudaMemcpyAsync(f_out + (size_t)s0 * pitch, dev64(c), n * sizeof(double),
                         cudaMemcpyDeviceToHost, r->copy_stream));
    else
      CK(cudaMemcpy2DAsync(f_out + (size_t)s0 * pitch, pitch * sizeof(double), dev64(c), row,
                           row, (size_t)(s1 - s0), cudaMemcpyDeviceToHost, r->copy_stream));
  }
  CK(cudaStreamSynchronize(r->copy_stream));
  if (rc) return rc;
  return check_status(r, false, nullptr);
}

extern "C" void *eprem_gpu_host_alloc(size_t bytes) {
  void *p = nullptr;
  if (cudaMallocHost(&p, bytes ? bytes : 1) != cudaSuccess) {
    fail(EPREM_GPU_ERR_CUDA, "page-locked host allocation failed");
    return nullptr;
  }
  return p;
}

extern "C" void eprem_gpu_host_free(void *p) {
  if (p) cudaFreeHost(p);
}

extern "C" int eprem_gpu_host_register(void *p, size_t bytes) {
  if (!p || !bytes) return fail(EPREM_GPU_ERR_ARG, "null argument");
  CK(cudaHostRegister(p, bytes, cudaHostRegisterDefault));
  return EPREM_GPU_OK;
}

extern "C" int eprem_gpu_host_unregister(void *p) {
  if (!p) return fail(EPREM_GPU_ERR_ARG, "null argument");
  CK(cudaHostUnregister(p));
  return EPREM_GPU_OK;
}

extern "C" int eprem_gpu_read_stats(eprem_gpu_run *r, eprem_ep_stats_t *stats) {
  if (!r || !stats) return fail(EPREM_GPU_ERR_ARG, "null argument");
  return check_status(r, true, stats);
}

extern "C" int eprem_gpu_update_mhd(eprem_gpu_run *r, double t_global) {
  if (!r) return fail(EPREM_GPU_ERR_ARG, "null run");
  if (r->mas_on && r->drift_on)
    return fail(EPREM_GPU_ERR_UNSUPPORTED,
                "drift with the MAS background (masGetNode does not form curl(B)/B^2)");
  if (r->mas_on) {
    if (!r->mas_selected)
      return fail(EPREM_GPU_ERR_STATE, "MAS background: no time slices selected");
    if (timed(r, EPREM_KERNEL_MHD, [&] {
          return launch_mas_update_mhd(r->v, r->mv, r->params.t_del, r->stream, &r->launches);
        }))
      return cuda_fail(cudaGetLastError(), "updateMhd (MAS) launch");
    return mas_mark_used(r);
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
  for (cudaEvent_t ev : r->mas_ready_ev) cudaEventDestroy(ev);
  for (cudaEvent_t ev : r->mas_used_ev) cudaEventDestroy(ev);
  r->mas_ready_ev.assign(mp->max_slices, nullptr);
  r->mas_used_ev.assign(mp->max_slices, nullptr);
  r->mas_pending.assign(mp->max_slices, 0);
  r->mas_used.assign(mp->max_slices, 0);
  r->mas_sel[0] = r->mas_sel[1] = -1;
  r->mv.radial_max = mp->radial_max;
  r->mv.v_min = mp->v_min;
  r->mv.cor_rotate_fake = mp->cor_rotate_fake;
  r->mv.rotate_solution = mp->rotate_solution;
  r->mv.r_scale = r->params.r_scale;
  r->mv.omega_sun = r->params.omega_sun;
  return EPREM_GPU_OK;
}

// One slice into device slot `slot`.  The slot's device arrays are kept
// from load to load while the slice's dimensions stay the same (a MAS run
// keeps one grid), so later loads allocate nothing.  async: the copies run
// on the run's copy stream after the slot's last reader, and selecting the
// slot makes the run's stream wait for them; otherwise they run on the run's
// stream and the call returns once they are done.
static int mas_store(eprem_gpu_run *r, int slot, const eprem_mas_slice_t *s, bool async) {
  if (!r || !s) return fail(EPREM_GPU_ERR_ARG, "null argument");
  if (!r->mas_ready) return fail(EPREM_GPU_ERR_STATE, "eprem_gpu_mas_init first");
  if (slot < 0 || slot >= (int)r->mas_slots.size()) return fail(EPREM_GPU_ERR_ARG, "slot out of range");
  if (async && (slot == r->mas_sel[0] || slot == r->mas_sel[1]))
    return fail(EPREM_GPU_ERR_STATE, "an asynchronous load needs a slot that is not selected");
  for (int f = 0; f < EPREM_MAS_NFIELDS; f++) {
    if (!s->data[f]) return fail(EPREM_GPU_ERR_ARG, "null MAS field");
    for (int a = 0; a < 3; a++)
      if (s->dims[f][a] < 2 || !s->mesh[f][a])
        return fail(EPREM_GPU_ERR_ARG, "MAS meshes need >= 2 points");
  }
  MasSlotDev &dev = r->mas_slots[slot];
  bool same = !r->mas_allocs[slot].empty();
  for (int f = 0; f < EPREM_MAS_NFIELDS && same; f++)
    for (int a = 0; a < 3; a++) same = same && dev.dims[f][a] == s->dims[f][a];
  if (!r->mas_ready_ev[slot]) {
    CK(cudaEventCreateWithFlags(&r->mas_ready_ev[slot], cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&r->mas_used_ev[slot], cudaEventDisableTiming));
  }
  if (async && !r->copy_stream) {
    CK(cudaStreamCreateWithFlags(&r->copy_stream, cudaStreamNonBlocking));
    for (cudaEvent_t &ev : r->stage_ev) CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  }
  if (!same) {  // first load of the slot, or a new grid: (re)allocate, nothing in flight
    CK(cudaStreamSynchronize(r->stream));
    if (r->copy_stream) CK(cudaStreamSynchronize(r->copy_stream));
    for (void *p : r->mas_allocs[slot]) cudaFree(p);
    r->mas_allocs[slot].clear();
    dev = MasSlotDev{};
    for (int f = 0; f < EPREM_MAS_NFIELDS; f++) {
      size_t n = 1;
      for (int a = 0; a < 3; a++) {
        float *m = nullptr;
        CK(cudaMalloc(&m, s->dims[f][a] * sizeof(float)));
        r->mas_allocs[slot].push_back(m);
        dev.mesh[f][a] = m;
        dev.dims[f][a] = s->dims[f][a];
        n *= (size_t)s->dims[f][a];
      }
      float *v = nullptr;
      CK(cudaMalloc(&v, n * sizeof(float)));
      r->mas_allocs[slot].push_back(v);
      dev.data[f] = v;
    }
  }
  r->mas_loaded[slot] = 0;
  cudaStream_t cs = async ? r->copy_stream : r->stream;
  if (async && r->mas_used[slot]) CK(cudaStreamWaitEvent(cs, r->mas_used_ev[slot], 0));
  for (int f = 0; f < EPREM_MAS_NFIELDS; f++) {
    size_t n = 1;
    for (int a = 0; a < 3; a++) {
      CK(cudaMemcpyAsync(const_cast<float *>(dev.mesh[f][a]), s->mesh[f][a],
                         s->dims[f][a] * sizeof(float), cudaMemcpyHostToDevice, cs));
      n *= (size_t)s->dims[f][a];
    }
    CK(cudaMemcpyAsync(const_cast<float *>(dev.data[f]), s->data[f], n * sizeof(float),
                       cudaMemcpyHostToDevice, cs));
  }
  if (async) {
    CK(cudaEventRecord(r->mas_ready_ev[slot], cs));
    r->mas_pending[slot] = 1;
  } else {
    CK(cudaStreamSynchronize(cs));
    r->mas_pending[slot] = 0;
  }
  r->mas_loaded[slot] = 1;
  return EPREM_GPU_OK;
}

extern "C" int eprem_gpu_mas_load_slice(eprem_gpu_run *r, int slot, const eprem_mas_slice_t *s) {
  return mas_store(r, slot, s, false);
}

extern "C" int eprem_gpu_mas_load_slice_async(eprem_gpu_run *r, int slot,
                                              const eprem_mas_slice_t *s) {
  return mas_store(r, slot, s, true);
}

// After a launch that reads the selected slots: mark them read (an async
// load into either waits for this point of the run's stream).
static int mas_mark_used(eprem_gpu_run *r) {
  for (int i = 0; i < 2; i++) {
    const int sl = r->mas_sel[i];
    if (sl < 0) continue;
    CK(cudaEventRecord(r->mas_used_ev[sl], r->stream));
    r->mas_used[sl] = 1;
  }
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
  for (int sl : {slot0, slot1})
    if (r->mas_pending[sl]) {  // an asynchronous load: the run's stream waits for its copies
      CK(cudaStreamWaitEvent(r->stream, r->mas_ready_ev[sl], 0));
      r->mas_pending[sl] = 0;
    }
  r->mv.s0 = r->mas_slots[slot0];
  r->mv.s1 = r->mas_slots[slot1];
  r->mv.s_cor = s_cor;
  r->mv.phi_offset = phi_offset;
  r->mas_sel[0] = slot0;
  r->mas_sel[1] = slot1;
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
  return mas_mark_used(r);
}

extern "C" int eprem_gpu_move_nodes(eprem_gpu_run *r, double dt) {
  if (!r) return fail(EPREM_GPU_ERR_ARG, "null run");
  if (timed(r, EPREM_KERNEL_MOVE,
            [&] { return launch_move_nodes(r->v, dt, r->stream, &r->launches); }))
    return cuda_fail(cudaGetLastError(), "moveNodes launch");
  return EPREM_GPU_OK;
}

extern "C" int eprem_gpu_set_time_step(eprem_gpu_run *r, double t_del) {
  if (!r) return fail(EPREM_GPU_ERR_ARG, "null run");
  if (!(t_del > 0.0) || !std::isfinite(t_del)) return fail(EPREM_GPU_ERR_ARG, "t_del must be finite and > 0");
  // every launch takes the run view by value: later launches see the new step
  r->params.t_del = t_del;
  r->v.dt = t_del / (1.0 * r->params.num_ep_steps);  // src/energeticParticles.c:99
  r->v.dt_full = r->v.dt * r->params.num_ep_steps;
  r->mhd.t_del = t_del;
  return EPREM_GPU_OK;
}

// The second f buffer (and its row exponents) that a perpendicular step
// writes before it becomes the run's f.
static int ensure_second_f(eprem_gpu_run *r) {
  if (r->d_shell_f) return EPREM_GPU_OK;
  const size_t elem = r->dims.precision == EPREM_FP32 ? sizeof(float) : sizeof(double);
  CK(cudaMalloc(&r->d_shell_f, elem * r->cells() + 16));  // as d_f, tail zeroed as there
  CK(cudaMemset(r->d_shell_f, 0, elem * r->cells() + 16));
  if (r->dims.precision == EPREM_FP32) {
    CK(cudaMalloc(&r->d_shell_fexp, sizeof(short) * r->sn() * r->dims.num_energies + 16));
    CK(cudaMemset(r->d_shell_fexp, 0, sizeof(short) * r->sn() * r->dims.num_energies));
  }
  return EPREM_GPU_OK;
}

// Per target stream, the NEWS hand-overs it receives in the reference's
// order (source streams ascending, per source north, east, west, south);
// with per_direction_loss (DriftShellData) each direction of the target's
// own row adds its loss right after that direction's gain, else
// (DiffuseShellData) one summed loss follows the target's four directions.
// Rows padded with -1 to the longest; *L its length.
static std::vector<int> news_gather_lists(const int32_t *news, int S, bool per_direction_loss,
                                          int *L) {
  std::vector<std::vector<int>> lists(S);
  for (int i = 0; i < S; i++) {
    for (int d = 0; d < 4; d++) {
      lists[news[i * 4 + d]].push_back(i * 8 + d);
      if (per_direction_loss) lists[i].push_back(i * 8 + 4 + d);
    }
    if (!per_direction_loss) lists[i].push_back(i * 8 + 4);
  }
  size_t n = 0;
  for (const auto &l : lists) n = std::max(n, l.size());
  std::vector<int> ent(n * S, -1);
  for (int j = 0; j < S; j++) std::copy(lists[j].begin(), lists[j].end(), ent.begin() + j * n);
  *L = (int)n;
  return ent;
}

extern "C" int eprem_gpu_set_drift(eprem_gpu_run *r, const int32_t *news,
                                   const eprem_drift_params_t *dp) {
  if (!r) return fail(EPREM_GPU_ERR_ARG, "null run");
  CK(cudaStreamSynchronize(r->stream));  // earlier launches may read what changes here
  if (!dp) {
    r->drift_on = false;
    r->v.curl = nullptr;
    return EPREM_GPU_OK;
  }
  if (r->mas_on)
    return fail(EPREM_GPU_ERR_UNSUPPORTED,
                "drift with the MAS background (masGetNode does not form curl(B)/B^2)");
  if (!(dp->mass > 0.0) || !std::isfinite(dp->charge) || dp->charge == 0.0 ||
      !std::isfinite(dp->lnpmin))
    return fail(EPREM_GPU_ERR_ARG, "drift: charge non-zero, mass > 0 and lnpmin finite");
  const int S = r->dims.num_streams, E = r->dims.num_energies;
  if (news)
    for (int i = 0; i < 4 * S; i++)
      if (news[i] < 0 || news[i] >= S) return fail(EPREM_GPU_ERR_ARG, "NEWS neighbour out of range");
  // driftVelocity's energy factor (src/energeticParticles.c:222-226), host libm
  const double mhd_b_norm = sqrt(kMp * kMhdDensityNorm) * kC;  // MHD_B_NORM
  const double om = mhd_b_norm * kQ * kAu / (kMp * kC * kC);    // OM, src/baseTypes.h:98
  const double om1 = dp->charge * om / dp->mass;
  for (int e = 0; e < E; e++) {
    const double p = exp(dp->lnpmin + e * r->grid_dlnp);
    r->h_ec[e].drift_factor = (1.0 / om1) * (p * r->h_ec[e].vgrid / 3.0);
  }
  CK(cudaMemcpy(r->d_ec, r->h_ec.data(), E * sizeof(EnergyConsts), cudaMemcpyHostToDevice));
  if (!r->d_curl) {
    CK(cudaMalloc(&r->d_curl, sizeof(double) * 3 * r->sn()));
    CK(cudaMemset(r->d_curl, 0, sizeof(double) * 3 * r->sn()));
  }
  r->v.curl = r->d_curl;
  r->drift_on = true;
  if (news) {
    int L = 0;
    const std::vector<int> ent = news_gather_lists(news, S, true, &L);
    if (!r->d_drift_news) {
      CK(cudaMalloc(&r->d_drift_news, sizeof(int) * 4 * (size_t)S));
      const size_t elem = r->dims.precision == EPREM_FP32 ? sizeof(float) : sizeof(double);
      CK(cudaMalloc(&r->d_drift_del, elem * 4 * r->sn() * E));
    }
    const int rc = ensure_second_f(r);
    if (rc) return rc;
    cudaFree(r->d_drift_ent);
    r->d_drift_ent = nullptr;
    CK(cudaMalloc(&r->d_drift_ent, sizeof(int) * ent.size()));
    CK(cudaMemcpy(r->d_drift_news, news, sizeof(int) * 4 * (size_t)S, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(r->d_drift_ent, ent.data(), sizeof(int) * ent.size(), cudaMemcpyHostToDevice));
    r->drift_L = L;
    r->drift_links = true;
  }
  return EPREM_GPU_OK;
}

extern "C" int eprem_gpu_set_shell_diffusion(eprem_gpu_run *r, const int32_t *news,
                                             double kperxkpar) {
  if (!r) return fail(EPREM_GPU_ERR_ARG, "null run");
  int rc = EPREM_GPU_OK;
  if (!news) {
    r->shell_on = false;
    return EPREM_GPU_OK;
  }
  const int S = r->dims.num_streams;
  // configuration.c reads kperxkpar with a lower bound of VERYSMALL
  if (!(kperxkpar >= kVerySmall) || !std::isfinite(kperxkpar))
    return fail(EPREM_GPU_ERR_ARG, "kperxkpar must be finite and >= 1e-33");
  for (int i = 0; i < 4 * S; i++)
    if (news[i] < 0 || news[i] >= S) return fail(EPREM_GPU_ERR_ARG, "NEWS neighbour out of range");
  // Per target stream, its incoming terms in the reference's order: source
  // streams ascending and, per source, north, east, west, south, then the
  // source's own loss (entry source * 8 + 4); rows padded to the longest.
  int L = 0;
  const std::vector<int> ent = news_gather_lists(news, S, false, &L);
  CK(cudaStreamSynchronize(r->stream));  // earlier launches may read the old lists
  if (!r->d_news) {
    CK(cudaMalloc(&r->d_news, sizeof(int) * 4 * (size_t)S));
    CK(cudaMalloc(&r->d_shell_del, sizeof(double) * 5 * r->sn() * r->dims.num_energies));
  }
  rc = ensure_second_f(r);
  if (rc) return rc;
  cudaFree(r->d_shell_ent);
  r->d_shell_ent = nullptr;
  CK(cudaMalloc(&r->d_shell_ent, sizeof(int) * ent.size()));
  CK(cudaMemcpy(r->d_news, news, sizeof(int) * 4 * (size_t)S, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(r->d_shell_ent, ent.data(), sizeof(int) * ent.size(), cudaMemcpyHostToDevice));
  r->shell_L = (int)L;
  r->kperxkpar = kperxkpar;
  r->shell_on = true;
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
// file-scope device array of this file's module; with lazy module loading
// the module -- and the buffer -- becomes resident when its address is first
// looked up, which eprem_gpu_create does for its device (with that device
// current) before it allocates anything, so the entry point itself never
// loads or allocates.  Every value is written by the flux kernel before it is
// copied out, so no part of the buffer needs zeroing.  All runs on a device
// share it: calls that overlap in time race on it and must be serialised by
// the caller.
namespace {
__device__ __align__(256) double g_flux_static[EPREM_GPU_FLUX_STATIC_MAX];
std::mutex g_flux_static_mutex;
double *g_flux_static_addr[kMaxDevices] = {};

// device: the current device (the caller makes it so)
int flux_static_buffer(int device, double **out) {
  if (device < 0 || device >= kMaxDevices)
    return fail(EPREM_GPU_ERR_ARG, "device ordinal beyond the static flux buffer table");
  std::lock_guard<std::mutex> lock(g_flux_static_mutex);
  if (!g_flux_static_addr[device]) {
    void *addr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&addr, g_flux_static);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(static flux buffer)");
    g_flux_static_addr[device] = static_cast<double *>(addr);
  }
  *out = g_flux_static_addr[device];
  return EPREM_GPU_OK;
}
}  // namespace

extern "C" int eprem_gpu_omni_flux_static(eprem_gpu_run *r, double *out) {
  if (!r || !out) return fail(EPREM_GPU_ERR_ARG, "null argument");
  int current = -1;
  CK(cudaGetDevice(&current));
  if (current != r->device)
    return fail(EPREM_GPU_ERR_ARG, "eprem_gpu_omni_flux_static: make the run's device current");
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

