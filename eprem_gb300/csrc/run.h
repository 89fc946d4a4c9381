// run.h -- private to the ABI layer (eprem_gpu.cu, ensemble.cu,
// surrogate_host.cu): the state behind an eprem_gpu_run handle and the error
// helpers every entry point uses.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/eprem_gpu.h"
#include "common.cuh"
#include "kernels.h"

namespace eprem {

// Failure of the calling thread's last ABI call (eprem_gpu_last_error).
int fail(int code, const std::string &msg);
int cuda_fail(cudaError_t e, const char *what);
constexpr int kMaxDevices = 64;  // per-device tables (static buffers, error flags)

}  // namespace eprem

#define CK(call)                                                  \
  do {                                                            \
    cudaError_t _e = (call);                                      \
    if (_e != cudaSuccess) return eprem::cuda_fail(_e, #call);    \
  } while (0)

struct eprem_gpu_run {
  eprem_dims_t dims;
  eprem_params_t params;
  int device = 0;
  cudaStream_t stream = nullptr;
  eprem::RunView v{};
  eprem::MhdParams mhd{};
  eprem::StreamPlan splan{};
  std::string skernel;  // eprem_gpu_stream_kernel's text
  eprem::NodePlan nplan{};
  int m0 = 0;
  double norm_radius = 0, neg_beta = 0;
  double grid_dlnp = 0;  // dlnp of the momentum grid
  void *d_f = nullptr;
  short *d_fexp = nullptr;  // FP32 form: row exponents [S][N][E]
  double *d_nodes = nullptr, *d_mugrid = nullptr;
  float *d_mugrid32 = nullptr;
  eprem::NodeCoef32 *d_coef32 = nullptr;
  float4 *d_scoef = nullptr;
  eprem::EnergyConsts *d_ec = nullptr;
  int *d_list = nullptr, *d_list_size = nullptr;
  double *d_ds_i = nullptr, *d_ds_min = nullptr, *d_seed_radial = nullptr, *d_mfp_node = nullptr;
  eprem::DevStatus *d_status = nullptr, *h_status = nullptr;
  // FP32 form: two staging buffers of FP64 chunks; downloads copy to the
  // host on their own stream, overlapping the conversion of the other buffer
  double *d_stage = nullptr;  // [2][stage_elems]
  size_t stage_elems = 0;
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t stage_ev[4] = {};  // converted[2], copied[2]
  double *d_flux = nullptr;
  double *d_tmpl = nullptr;   // [S][E][M] template rows of eprem_gpu_ripple_f
  // shell diffusion (eprem_gpu_set_shell_diffusion): NEWS links, per-target
  // gather lists (S x shell_L, padded with -1), per-call fractions and a
  // second f buffer that each diffusion step writes and then swaps with d_f
  bool shell_on = false;
  double kperxkpar = 0.0;
  int shell_L = 0;
  int *d_news = nullptr, *d_shell_ent = nullptr;
  void *d_shell_del = nullptr;    // Real[N][E][S][5]
  void *d_shell_f = nullptr;      // Real[S][N][E][M]
  short *d_shell_fexp = nullptr;  // FP32 form: its row exponents
  // drift (eprem_gpu_set_drift): curl(B)/B^2 per node, the drift NEWS links,
  // per-target gather lists (S x drift_L) and per-call fractions
  bool drift_on = false, drift_links = false;
  double *d_curl = nullptr;       // [3][S*N]
  int *d_drift_news = nullptr, *d_drift_ent = nullptr;
  int drift_L = 0;
  void *d_drift_del = nullptr;    // Real[N][E][S][4]
  std::vector<eprem::EnergyConsts> h_ec;  // host copy of d_ec
  uint64_t launches = 0;
  // optional per-launch timing: events recorded around each kernel launch
  bool timing = false;
  std::vector<cudaEvent_t> ev_pool;
  std::vector<std::pair<int, int>> ev_pending;  // (kind, index of start event)
  size_t ev_used = 0;
  // node phase: reference, split or surrogate (EPREM_NODE_PHASE_*)
  int node_mode = 0;
  struct eprem_gpu_surrogate *surr = nullptr;
  unsigned long long *d_surr_counts = nullptr;  // [kept, fallback] rows
  uint8_t *d_reject = nullptr;
  // MAS background: device copies of the loaded time slices
  bool mas_ready = false;  // eprem_gpu_mas_init done
  bool mas_on = false, mas_selected = false;  // updateMhd uses MAS; slots chosen
  std::vector<std::vector<void *>> mas_allocs;
  std::vector<eprem::MasSlotDev> mas_slots;
  std::vector<char> mas_loaded;
  // per slot: copy done (async loads, on copy_stream) and last read (on stream)
  std::vector<cudaEvent_t> mas_ready_ev, mas_used_ev;
  std::vector<char> mas_pending, mas_used;
  int mas_sel[2] = {-1, -1};
  eprem::MasView mv{};
  size_t cells() const {
    return (size_t)dims.num_streams * dims.num_nodes * dims.num_energies * dims.num_mu;
  }
  size_t sn() const { return (size_t)dims.num_streams * dims.num_nodes; }
};

namespace eprem {

// Runs one launch helper, bracketed by events when timing is on.
template <typename Fn>
inline int timed(eprem_gpu_run *r, int kind, Fn &&launch) {
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

// Reads the status block (synchronising), reports a device failure in the
// reference's words and, with reset_stats, hands over and restarts the log
// statistics.
int check_status(eprem_gpu_run *r, bool reset_stats, eprem_ep_stats_t *stats);
// The node phase of one EP sub-step in the split and surrogate forms.
int split_node_phase(eprem_gpu_run *r);
// updateEnergeticParticles in pieces, on the run's stream: the per-call
// set-up, then per EP sub-step the streaming (or seed check) and the node
// phase with the perpendicular steps.
int ep_begin(eprem_gpu_run *r, const RunView &v);
int ep_stream_phase(eprem_gpu_run *r, const RunView &v);
int ep_node_phase(eprem_gpu_run *r, const RunView &v);

}  // namespace eprem
