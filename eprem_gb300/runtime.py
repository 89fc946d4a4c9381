"""Host-side mirror of the reference's hot-path entry points over the C ABI.

The reference drives the path through argument-less C functions acting on
globals (updateEnergeticParticles, updateMhd, moveNodes; see
include/eprem_gpu.h).  ``EpremRun`` keeps the same verbs, backed by
libeprem_gpu.so through ctypes: state is uploaded once, the verbs run on the
GPU, and results are downloaded when the caller asks.

There is no CPU fallback: if the CUDA library is missing or no GPU is present,
construction raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libeprem_gpu.so")
DP = C.POINTER(C.c_double)
FP = C.POINTER(C.c_float)

# Every entry point of include/eprem_gpu.h: (name, restype, argtypes)
EXPORTS = [
    ("eprem_gpu_create", C.c_int,
     [C.POINTER(abi.Dims), C.POINTER(abi.Params), C.POINTER(abi.Grids), C.POINTER(C.c_void_p)]),
    ("eprem_gpu_destroy", C.c_int, [C.c_void_p]),
    ("eprem_gpu_upload_f", C.c_int, [C.c_void_p, DP]),
    ("eprem_gpu_download_f", C.c_int, [C.c_void_p, DP]),
    ("eprem_gpu_upload_nodes", C.c_int, [C.c_void_p, DP, C.c_uint64]),
    ("eprem_gpu_download_nodes", C.c_int, [C.c_void_p, DP, C.c_uint64]),
    ("eprem_gpu_update_energetic_particles", C.c_int, [C.c_void_p, C.c_double]),
    ("eprem_gpu_read_stats", C.c_int, [C.c_void_p, C.POINTER(abi.EpStats)]),
    ("eprem_gpu_update_mhd", C.c_int, [C.c_void_p, C.c_double]),
    ("eprem_gpu_move_nodes", C.c_int, [C.c_void_p, C.c_double]),
    ("eprem_gpu_set_time_step", C.c_int, [C.c_void_p, C.c_double]),
    ("eprem_gpu_surrogate_calibrate_error", C.c_int,
     [C.c_void_p, C.c_double, C.c_int64, C.POINTER(C.c_double), C.POINTER(C.c_double),
      C.POINTER(C.c_double)]),
    ("eprem_gpu_set_drift", C.c_int,
     [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(abi.DriftParams)]),
    ("eprem_gpu_set_shell_diffusion", C.c_int,
     [C.c_void_p, C.POINTER(C.c_int32), C.c_double]),
    ("eprem_gpu_update_energetic_particles_host", C.c_int,
     [C.c_void_p, DP, DP, C.c_size_t, C.c_double]),
    ("eprem_gpu_host_alloc", C.c_void_p, [C.c_size_t]),
    ("eprem_gpu_host_free", None, [C.c_void_p]),
    ("eprem_gpu_host_register", C.c_int, [C.c_void_p, C.c_size_t]),
    ("eprem_gpu_upload_f_pitched", C.c_int, [C.c_void_p, DP, C.c_size_t]),
    ("eprem_gpu_download_f_pitched", C.c_int, [C.c_void_p, DP, C.c_size_t]),
    ("eprem_gpu_ripple_f", C.c_int, [C.c_void_p, DP, C.c_size_t]),
    ("eprem_gpu_host_unregister", C.c_int, [C.c_void_p]),
    ("eprem_gpu_omni_flux", C.c_int, [C.c_void_p, DP]),
    ("eprem_gpu_omni_flux_static", C.c_int, [C.c_void_p, DP]),
    ("eprem_gpu_synchronize", C.c_int, [C.c_void_p]),
    ("eprem_gpu_stream", C.c_void_p, [C.c_void_p]),
    ("eprem_gpu_kernel_launches", C.c_uint64, [C.c_void_p]),
    ("eprem_gpu_set_kernel_timing", C.c_int, [C.c_void_p, C.c_int]),
    ("eprem_gpu_read_kernel_timing", C.c_int, [C.c_void_p, C.POINTER(abi.KernelTime)]),
    ("eprem_gpu_alu_peak", C.c_int, [C.c_int, DP]),
    ("eprem_gpu_mas_init", C.c_int, [C.c_void_p, C.POINTER(abi.MasParams)]),
    ("eprem_gpu_mas_load_slice", C.c_int, [C.c_void_p, C.c_int, C.POINTER(abi.MasSlice)]),
    ("eprem_gpu_mas_load_slice_async", C.c_int, [C.c_void_p, C.c_int, C.POINTER(abi.MasSlice)]),
    ("eprem_gpu_mas_select", C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_double]),
    ("eprem_gpu_mas_move_nodes", C.c_int, [C.c_void_p, C.c_double]),
    ("eprem_gpu_mas_use", C.c_int, [C.c_void_p, C.c_int]),
    ("eprem_gpu_init_seed_population", C.c_int, [C.c_void_p, C.c_uint64, C.c_double]),
    ("eprem_gpu_autotune", C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    ("eprem_gpu_set_stream_variant", C.c_int, [C.c_void_p, C.c_int]),
    ("eprem_gpu_stream_kernel", C.c_char_p, [C.c_void_p]),
    ("eprem_gpu_plan_stream", C.c_int,
     [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int)]),
    ("eprem_gpu_ensemble_create", C.c_int, [C.POINTER(C.c_void_p), C.c_int,
                                            C.POINTER(C.c_void_p)]),
    ("eprem_gpu_ensemble_destroy", C.c_int, [C.c_void_p]),
    ("eprem_gpu_ensemble_set_time", C.c_int, [C.c_void_p, DP]),
    ("eprem_gpu_ensemble_get_time", C.c_int, [C.c_void_p, DP]),
    ("eprem_gpu_ensemble_autotune", C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    ("eprem_gpu_ensemble_set_chains", C.c_int, [C.c_void_p, C.c_int]),
    ("eprem_gpu_ensemble_step", C.c_int, [C.c_void_p]),
    ("eprem_gpu_ensemble_synchronize", C.c_int, [C.c_void_p]),
    ("eprem_gpu_ensemble_stream", C.c_void_p, [C.c_void_p]),
    ("eprem_gpu_gemm_bf16", C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p,
                                      C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int,
                                      C.c_void_p]),
    ("eprem_gpu_surrogate_create", C.c_int, [C.c_uint64, C.c_int, C.POINTER(C.c_void_p)]),
    ("eprem_gpu_surrogate_destroy", C.c_int, [C.c_void_p]),
    ("eprem_gpu_surrogate_num_params", C.c_int64, []),
    ("eprem_gpu_surrogate_get_params", C.c_int, [C.c_void_p, FP, C.c_int64]),
    ("eprem_gpu_surrogate_set_params", C.c_int, [C.c_void_p, FP, C.c_int64]),
    ("eprem_gpu_surrogate_reserve", C.c_int, [C.c_void_p, C.c_int64]),
    ("eprem_gpu_surrogate_collect", C.c_int, [C.c_void_p, C.c_void_p, C.c_double, C.c_uint64,
                                              C.POINTER(C.c_int64)]),
    ("eprem_gpu_surrogate_train", C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_double,
                                            C.POINTER(C.c_double)]),
    ("eprem_gpu_surrogate_loss_grad", C.c_int, [C.c_void_p, FP, FP, C.c_int,
                                                C.POINTER(C.c_double), FP]),
    ("eprem_gpu_surrogate_evaluate", C.c_int, [C.c_void_p, FP, C.c_int, FP]),
    ("eprem_gpu_surrogate_calibrate", C.c_int, [C.c_void_p, C.c_double, C.c_double,
                                                C.POINTER(C.c_double)]),
    ("eprem_gpu_surrogate_set_tolerance", C.c_int, [C.c_void_p, C.c_double]),
    ("eprem_gpu_set_node_phase", C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    ("eprem_gpu_surrogate_counts", C.c_int, [C.c_void_p, C.POINTER(C.c_uint64),
                                             C.POINTER(C.c_uint64)]),
    ("eprem_gpu_last_error", C.c_char_p, []),
]

_lib = None


class EpremGpuError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{abi.STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


def load_library(path: str = LIB_PATH):
    """Load libeprem_gpu.so (raises if it has not been built)."""
    global _lib
    if _lib is not None and path == LIB_PATH:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(
            f"{path} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(path)
    for name, res, args in EXPORTS:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path == LIB_PATH:
        _lib = lib
    return lib


def alu_peak_tflops(precision: int) -> float:
    """Measured FMA throughput (TFLOP/s) of the current GPU."""
    lib = load_library()
    out = C.c_double()
    rc = lib.eprem_gpu_alu_peak(precision, C.byref(out))
    if rc:
        raise EpremGpuError(rc, lib.eprem_gpu_last_error().decode())
    return out.value


def plan_stream(num_nodes: int, num_mu: int, m0: int, precision: int, variant: int = 0,
                seed_boundary: bool = True) -> dict:
    """The streaming kernel a run of these sizes would launch (host only, no
    device needed): kind, mu bin, threads, list nodes per thread, cluster
    size and the nodes a cluster holds."""
    lib = load_library()
    out = (C.c_int * 6)()
    rc = lib.eprem_gpu_plan_stream(num_nodes, num_mu, m0, precision, variant,
                                   1 if seed_boundary else 0, out)
    if rc:
        raise EpremGpuError(rc, lib.eprem_gpu_last_error().decode())
    return dict(zip(("kind", "mmax", "threads", "npt", "cluster", "slots"), list(out)))


def _dp(a: np.ndarray):
    if a.dtype != np.float64 or not a.flags["C_CONTIGUOUS"]:
        raise ValueError("expected a C-contiguous float64 array")
    return a.ctypes.data_as(DP)


class EpremRun:
    """One set of streams resident on the current GPU."""

    def __init__(self, dims: abi.Dims, params: abi.Params, grids: dict):
        self.lib = load_library()
        self.dims = dims
        self.params = params
        self._grids_keep = {k: np.ascontiguousarray(grids[k], dtype=np.float64)
                            for k in ("egrid", "vgrid", "vgrid_i", "mugrid", "rigidity")}
        g = abi.Grids(*(self._grids_keep[k].ctypes.data_as(DP)
                        for k in ("egrid", "vgrid", "vgrid_i", "mugrid", "rigidity")),
                      float(grids["dlnp"]), float(grids["dmu"]))
        h = C.c_void_p()
        self._check(self.lib.eprem_gpu_create(C.byref(dims), C.byref(params), C.byref(g),
                                              C.byref(h)))
        self.handle = h

    # -- helpers ------------------------------------------------------------
    def _check(self, rc: int):
        if rc != abi.EPREM_GPU_OK:
            raise EpremGpuError(rc, self.lib.eprem_gpu_last_error().decode())

    @property
    def num_cells(self) -> int:
        d = self.dims
        return d.num_streams * d.num_nodes * d.num_energies * d.num_mu

    @property
    def num_nodes_total(self) -> int:
        return self.dims.num_streams * self.dims.num_nodes

    def close(self):
        if getattr(self, "handle", None):
            self.lib.eprem_gpu_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- state ---------------------------------------------------------------
    def upload_f(self, f: np.ndarray):
        assert f.size == self.num_cells
        self._check(self.lib.eprem_gpu_upload_f(self.handle, _dp(f)))

    def download_f(self, out: np.ndarray | None = None) -> np.ndarray:
        out = np.empty(self.num_cells) if out is None else out
        self._check(self.lib.eprem_gpu_download_f(self.handle, _dp(out)))
        return out

    def upload_nodes(self, nodes: np.ndarray, mask: int = abi.NODE_MASK_ALL):
        assert nodes.size == abi.NODE_NFIELDS * self.num_nodes_total
        self._check(self.lib.eprem_gpu_upload_nodes(self.handle, _dp(nodes), mask))

    def download_nodes(self, out: np.ndarray | None = None,
                       mask: int = abi.NODE_MASK_ALL) -> np.ndarray:
        out = (np.zeros((abi.NODE_NFIELDS, self.num_nodes_total)) if out is None else out)
        self._check(self.lib.eprem_gpu_download_nodes(self.handle, _dp(out), mask))
        return out

    # -- the reference's verbs ------------------------------------------------
    def update_energetic_particles(self, t_global: float = 0.0):
        """updateEnergeticParticles (src/energeticParticles.c:70-203)."""
        self._check(self.lib.eprem_gpu_update_energetic_particles(self.handle, t_global))

    def update_mhd(self, t_global: float):
        """updateMhd, analytic background (src/flow.c:36-154)."""
        self._check(self.lib.eprem_gpu_update_mhd(self.handle, t_global))

    def move_nodes(self, dt: float):
        """moveNodes (src/simCore.c:737-785)."""
        self._check(self.lib.eprem_gpu_move_nodes(self.handle, dt))

    def update_energetic_particles_host(self, f_in: np.ndarray, f_out: np.ndarray = None,
                                       t_global: float = 0.0, stream_pitch: int = 0) -> np.ndarray:
        """updateEnergeticParticles with f in host memory, copies overlapped
        with the update chunk by chunk.  Stream s's N*E*M values start at
        element s * stream_pitch (0: N*E*M, contiguous).  f_out may be f_in;
        page-locked memory lets the copies overlap."""
        d = self.dims
        per_stream = d.num_nodes * d.num_energies * d.num_mu
        pitch = stream_pitch or per_stream
        need = (d.num_streams - 1) * pitch + per_stream
        assert f_in.dtype == np.float64 and f_in.size >= need and f_in.flags["C_CONTIGUOUS"]
        if f_out is None:
            f_out = np.empty(need)
        assert f_out.dtype == np.float64 and f_out.size >= need and f_out.flags["C_CONTIGUOUS"]
        self._check(self.lib.eprem_gpu_update_energetic_particles_host(
            self.handle, f_in.ctypes.data_as(DP), f_out.ctypes.data_as(DP), stream_pitch, t_global))
        return f_out

    def upload_f_pitched(self, f: np.ndarray, stream_pitch: int):
        """Upload f whose stream s starts at element s * stream_pitch."""
        assert f.dtype == np.float64 and f.flags["C_CONTIGUOUS"]
        self._check(self.lib.eprem_gpu_upload_f_pitched(self.handle, f.ctypes.data_as(DP),
                                                        stream_pitch))

    def download_f_pitched(self, f: np.ndarray, stream_pitch: int):
        assert f.dtype == np.float64 and f.flags["C_CONTIGUOUS"]
        self._check(self.lib.eprem_gpu_download_f_pitched(self.handle, f.ctypes.data_as(DP),
                                                          stream_pitch))

    def ripple_f(self, tmpl: np.ndarray, stream_pitch: int = 0):
        """rippleShellsOut for f: nodes move out by one, node 0 takes tmpl."""
        assert tmpl.dtype == np.float64 and tmpl.flags["C_CONTIGUOUS"]
        self._check(self.lib.eprem_gpu_ripple_f(self.handle, tmpl.ctypes.data_as(DP),
                                                stream_pitch))

    def set_time_step(self, t_del: float):
        """A new config.tDel from the next call on, as SetDT
        (src/simCore.c:800-880) sets it in MAS-coupled runs."""
        self._check(self.lib.eprem_gpu_set_time_step(self.handle, t_del))

    def set_shell_diffusion(self, news, kperxkpar: float = 0.01):
        """useShellDiffusion with config.kperxkpar: DiffuseShellData after
        every sub-step.  news: num_streams x 4 stream indices of each
        stream's north, east, west and south neighbour (None: off)."""
        if news is None:
            self._check(self.lib.eprem_gpu_set_shell_diffusion(self.handle, None, 0.0))
            return
        nw = np.ascontiguousarray(news, dtype=np.int32)
        if nw.shape != (self.dims.num_streams, 4):
            raise ValueError("news must be num_streams x 4")
        self._check(self.lib.eprem_gpu_set_shell_diffusion(
            self.handle, nw.ctypes.data_as(C.POINTER(C.c_int32)), kperxkpar))

    def set_drift(self, news, drift_params):
        """useDrift: curl(B)/B^2 formed by every analytic update_mhd and
        DriftShellData after every sub-step.  drift_params: abi.DriftParams
        (None: off); news: num_streams x 4 NEWS links (None keeps earlier
        ones)."""
        if drift_params is None:
            self._check(self.lib.eprem_gpu_set_drift(self.handle, None, None))
            return
        ptr = None
        if news is not None:
            nw = np.ascontiguousarray(news, dtype=np.int32)
            if nw.shape != (self.dims.num_streams, 4):
                raise ValueError("news must be num_streams x 4")
            self._drift_news = nw
            ptr = nw.ctypes.data_as(C.POINTER(C.c_int32))
        self._check(self.lib.eprem_gpu_set_drift(self.handle, ptr, C.byref(drift_params)))

    # -- MAS background ------------------------------------------------------
    def mas_init(self, mas_params: abi.MasParams):
        """Switch updateMhd to the MAS background (masGetNode)."""
        self._check(self.lib.eprem_gpu_mas_init(self.handle, C.byref(mas_params)))

    def mas_load_slice(self, slot: int, slice_struct: abi.MasSlice):
        self._check(self.lib.eprem_gpu_mas_load_slice(self.handle, slot, C.byref(slice_struct)))

    def mas_load_slice_async(self, slot: int, slice_struct: abi.MasSlice):
        """Queue the slice's copy on the run's copy stream (the arrays behind
        slice_struct must stay alive until the slot is next selected)."""
        self._check(self.lib.eprem_gpu_mas_load_slice_async(self.handle, slot,
                                                            C.byref(slice_struct)))

    def mas_select(self, slot0: int, slot1: int, s_cor: float, phi_offset: float = 0.0):
        self._check(self.lib.eprem_gpu_mas_select(self.handle, slot0, slot1, s_cor, phi_offset))

    def mas_use(self, use_mas: bool):
        """updateMhd's background after mas_init: MAS (True) or analytic."""
        self._check(self.lib.eprem_gpu_mas_use(self.handle, int(bool(use_mas))))

    def mas_move_nodes(self, dt: float):
        """masMoveNodes (src/masInterp.c:1344-1393)."""
        self._check(self.lib.eprem_gpu_mas_move_nodes(self.handle, dt))

    def read_stats(self) -> abi.EpStats:
        st = abi.EpStats()
        self._check(self.lib.eprem_gpu_read_stats(self.handle, C.byref(st)))
        return st

    def omni_flux(self) -> np.ndarray:
        d = self.dims
        out = np.empty(d.num_streams * d.num_nodes * d.num_energies)
        self._check(self.lib.eprem_gpu_omni_flux(self.handle, _dp(out)))
        return out

    def omni_flux_static(self) -> np.ndarray:
        """omni_flux staged in the library's fixed device buffer: allocates
        no device memory (S*N*E <= abi.FLUX_STATIC_MAX)."""
        d = self.dims
        out = np.empty(d.num_streams * d.num_nodes * d.num_energies)
        self._check(self.lib.eprem_gpu_omni_flux_static(self.handle, _dp(out)))
        return out

    def synchronize(self):
        self._check(self.lib.eprem_gpu_synchronize(self.handle))

    def set_kernel_timing(self, enable: bool):
        self._check(self.lib.eprem_gpu_set_kernel_timing(self.handle, int(enable)))

    def read_kernel_timing(self) -> dict:
        arr = (abi.KernelTime * len(abi.KERNEL_KINDS))()
        self._check(self.lib.eprem_gpu_read_kernel_timing(self.handle, arr))
        return {k: (arr[i].launches, arr[i].total_ms) for i, k in enumerate(abi.KERNEL_KINDS)}

    @property
    def stream(self) -> int:
        return self.lib.eprem_gpu_stream(self.handle)

    @property
    def kernel_launches(self) -> int:
        return int(self.lib.eprem_gpu_kernel_launches(self.handle))

    # -- synthetic state and tuning (no reference counterpart) ----------------
    def init_seed_population(self, seed: int, perturbation: float):
        """f = seed function x (1 + perturbation U(-1,1)) built on the device."""
        self._check(self.lib.eprem_gpu_init_seed_population(self.handle, int(seed),
                                                             float(perturbation)))

    def autotune(self) -> int:
        """Time the streaming shapes on a scratch copy and keep the fastest."""
        v = C.c_int()
        self._check(self.lib.eprem_gpu_autotune(self.handle, C.byref(v)))
        return v.value

    @property
    def stream_kernel(self) -> str:
        """The streaming kernel this run launches, with its shape."""
        return self.lib.eprem_gpu_stream_kernel(self.handle).decode()

    def set_stream_variant(self, variant: int):
        self._check(self.lib.eprem_gpu_set_stream_variant(self.handle, int(variant)))


class Ensemble:
    """Independent runs stepped together: one CUDA-graph launch per step
    (moveNodes, updateMhd at t + tDel, updateEnergeticParticles for every
    run).  The runs stay usable on their own after synchronize()."""

    def __init__(self, runs: list[EpremRun]):
        self.lib = load_library()
        self.runs = list(runs)
        arr = (C.c_void_p * len(runs))(*[r.handle.value for r in runs])
        h = C.c_void_p()
        self._check(self.lib.eprem_gpu_ensemble_create(arr, len(runs), C.byref(h)))
        self.handle = h

    def _check(self, rc: int):
        if rc != abi.EPREM_GPU_OK:
            raise EpremGpuError(rc, self.lib.eprem_gpu_last_error().decode())

    def set_time(self, t):
        t = np.ascontiguousarray(np.broadcast_to(np.asarray(t, dtype=np.float64),
                                                 (len(self.runs),)))
        self._check(self.lib.eprem_gpu_ensemble_set_time(self.handle, _dp(t)))

    def get_time(self) -> np.ndarray:
        out = np.empty(len(self.runs))
        self._check(self.lib.eprem_gpu_ensemble_get_time(self.handle, _dp(out)))
        return out

    def autotune(self) -> list[int]:
        out = (C.c_int * len(self.runs))()
        self._check(self.lib.eprem_gpu_ensemble_autotune(self.handle, out))
        return list(out)

    def set_chains(self, chains: int):
        """Graph schedule: `chains` serial chains side by side (1, the
        default: all runs in sequence; 0: one branch per run)."""
        self._check(self.lib.eprem_gpu_ensemble_set_chains(self.handle, chains))

    def step(self):
        self._check(self.lib.eprem_gpu_ensemble_step(self.handle))

    def synchronize(self):
        self._check(self.lib.eprem_gpu_ensemble_synchronize(self.handle))

    @property
    def stream(self) -> int:
        return self.lib.eprem_gpu_ensemble_stream(self.handle)

    def close(self):
        if getattr(self, "handle", None):
            self.lib.eprem_gpu_ensemble_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


NODE_PHASE_REFERENCE, NODE_PHASE_SPLIT, NODE_PHASE_SURROGATE, NODE_PHASE_SURROGATE_FOCUS = 0, 1, 2, 3


def _fp(a: np.ndarray):
    if a.dtype != np.float32 or not a.flags["C_CONTIGUOUS"]:
        raise ValueError("expected a C-contiguous float32 array")
    return a.ctypes.data_as(FP)


class Surrogate:
    """The learned focusing + scattering step (MLP 48-256-256-48, bf16 on
    the tensor cores): training set collection, training, calibration."""

    def __init__(self, seed: int = 1, chunk_rows: int = 0):
        self.lib = load_library()
        h = C.c_void_p()
        self._check(self.lib.eprem_gpu_surrogate_create(int(seed), int(chunk_rows), C.byref(h)))
        self.handle = h
        self.num_params = int(self.lib.eprem_gpu_surrogate_num_params())

    def _check(self, rc: int):
        if rc != abi.EPREM_GPU_OK:
            raise EpremGpuError(rc, self.lib.eprem_gpu_last_error().decode())

    def get_params(self) -> np.ndarray:
        out = np.empty(self.num_params, dtype=np.float32)
        self._check(self.lib.eprem_gpu_surrogate_get_params(self.handle, _fp(out), out.size))
        return out

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, dtype=np.float32)
        self._check(self.lib.eprem_gpu_surrogate_set_params(self.handle, _fp(p), p.size))

    def reserve(self, capacity: int):
        self._check(self.lib.eprem_gpu_surrogate_reserve(self.handle, int(capacity)))

    def collect(self, run: EpremRun, rate: float, seed: int) -> int:
        n = C.c_int64()
        self._check(self.lib.eprem_gpu_surrogate_collect(self.handle, run.handle, float(rate),
                                                         int(seed), C.byref(n)))
        return n.value

    def train(self, steps: int, batch: int = 8192, lr: float = 1e-3) -> float:
        loss = C.c_double()
        self._check(self.lib.eprem_gpu_surrogate_train(self.handle, int(steps), int(batch),
                                                       float(lr), C.byref(loss)))
        return loss.value

    def loss_grad(self, x: np.ndarray, t: np.ndarray):
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = np.ascontiguousarray(t, dtype=np.float32)
        g = np.empty(self.num_params, dtype=np.float32)
        loss = C.c_double()
        self._check(self.lib.eprem_gpu_surrogate_loss_grad(self.handle, _fp(x), _fp(t),
                                                           x.shape[0], C.byref(loss), _fp(g)))
        return loss.value, g

    def evaluate(self, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.empty((x.shape[0], 48), dtype=np.float32)
        self._check(self.lib.eprem_gpu_surrogate_evaluate(self.handle, _fp(x), x.shape[0],
                                                          _fp(y)))
        return y

    def calibrate(self, quantile: float = 0.999, margin: float = 1.5) -> float:
        tol = C.c_double()
        self._check(self.lib.eprem_gpu_surrogate_calibrate(self.handle, float(quantile),
                                                           float(margin), C.byref(tol)))
        return tol.value

    def calibrate_error(self, target: float, rows: int = 0):
        """Tolerance from the rows' true error against their plain step:
        (tolerance, fraction kept by the check, fraction within target)."""
        tol, kept, within = C.c_double(), C.c_double(), C.c_double()
        self._check(self.lib.eprem_gpu_surrogate_calibrate_error(
            self.handle, float(target), int(rows), C.byref(tol), C.byref(kept),
            C.byref(within)))
        return tol.value, kept.value, within.value

    def set_tolerance(self, tol: float):
        self._check(self.lib.eprem_gpu_surrogate_set_tolerance(self.handle, float(tol)))

    def close(self):
        if getattr(self, "handle", None):
            self.lib.eprem_gpu_surrogate_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def set_node_phase(run: EpremRun, mode: int, surrogate: Surrogate | None = None):
    lib = load_library()
    rc = lib.eprem_gpu_set_node_phase(run.handle, int(mode),
                                      surrogate.handle if surrogate is not None else None)
    if rc != abi.EPREM_GPU_OK:
        raise EpremGpuError(rc, lib.eprem_gpu_last_error().decode())


def surrogate_counts(run: EpremRun) -> tuple[int, int]:
    lib = load_library()
    k, f = C.c_uint64(), C.c_uint64()
    rc = lib.eprem_gpu_surrogate_counts(run.handle, C.byref(k), C.byref(f))
    if rc != abi.EPREM_GPU_OK:
        raise EpremGpuError(rc, lib.eprem_gpu_last_error().decode())
    return k.value, f.value
