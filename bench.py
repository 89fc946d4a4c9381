"""Benchmark of the GB300 energetic-particle update.

Metric: cell-updates/s, one cell-update = one (node, energy, mu) cell through
one EP sub-step (streaming + isotropisation, focusing, adiabatic change).  A
step is one driver step of the hot path: moveNodes + updateMhd +
updateEnergeticParticles (numEpSteps = 30 sub-steps), src/eprem.c:620-671.

Workload (default): the precision-at-scale case -- 1536 streams x 1000 nodes x
50 energies (0.1-1000 MeV) x 40 mu, Parker wind, seed power law -- in the
chosen form (f and stencil arithmetic in FP32, geometry / CFL in FP64).  The
plain FP64 form is measured beside it on a 96-stream subset with identical
per-stream work, and the FP32 omnidirectional flux is compared with it.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line (rank 0).  Under torchrun every rank runs its own
independent copy of the workload (streams are independent; no collective on
the data path), so scaling is weak.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "cell-updates/s (node*E*mu) plain FP64 vs chosen form at <=1e-3 rel flux err"
UNIT = "cell-updates/s"
FLOPS_PER_CELL_SUBCYCLE = {"stream": 8.0, "focus": 11.0, "change": 11.0}
BYTES_PER_CELL_UPDATE = {"fp64": 32.0, "fp32": 16.0}
# DRAM bytes (read + write) per cell per launch of the dominant kernel, from
# one ncu capture of the 96-stream subset (profiles/k_stream2_pairs_fp32_96streams.txt,
# profiles/k_stream_fp64_96streams.txt, profiles/k_focus32_k_change32_fp32_96streams.txt):
# traffic per launch / 96*1000*50*40 cells; traffic grows with the number of
# (stream, energy) slabs, so it scales to a full launch by the cells processed.
NCU_DRAM_BYTES_PER_CELL = {("stream", "fp32"): 1570.3949e6 / 192e6,
                           ("stream", "fp64"): 3054.831e6 / 192e6,
                           ("node", "fp32"): 1488.048e6 / 192e6}


# ---------------------------------------------------------------------------
def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["scale", "small"], default="scale")
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--fp64-faces", type=int, default=4,
                    help="rows=cols of the plain-FP64 subset (6*n*n streams)")
    ap.add_argument("--skip-fp64", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-mas", action="store_true")
    ap.add_argument("--skip-ensemble", action="store_true")
    ap.add_argument("--ensemble-runs", type=int, default=8,
                    help="members of the 64-run batched ensemble to step (first n)")
    ap.add_argument("--ensemble-steps", type=int, default=2)
    ap.add_argument("--ensemble-only", action="store_true",
                    help="measure only the batched ensemble (with --ensemble-runs 64: the full set)")
    ap.add_argument("--skip-surrogate", action="store_true")
    ap.add_argument("--surrogate-train-steps", type=int, default=4000)
    ap.add_argument("--mas-steps", type=int, default=2)
    ap.add_argument("--stream-variant", type=int, default=0,
                    help="streaming-kernel shape of the --profile-step run (0 automatic)")
    ap.add_argument("--profile-step", choices=["fp32", "fp64"], default=None,
                    help="run one EP sub-step of the 96-stream subset and exit "
                         "(the case the ncu captures use)")
    ap.add_argument("--shell-diffusion", type=float, default=None, metavar="KPERXKPAR",
                    help="with --profile-step: shell diffusion on (torus NEWS links, every "
                         "stream with four in-links as on the cube sphere); prints the "
                         "CUDA-event time of each kernel kind of the second of two steps")
    return ap.parse_args()


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return 0, 1, None
    import torch
    import torch.distributed as dist
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    rank = int(os.environ["RANK"])
    local = int(os.environ.get("LOCAL_RANK", rank))
    backend = "nccl" if torch.cuda.is_available() else "gloo"
    if backend == "nccl":
        torch.cuda.set_device(local)
    dist.init_process_group(backend)
    return rank, ws, dist


def reduce_max(dist, x: float) -> float:
    if dist is None:
        return x
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during a region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int = 0):
        self.index = index
        self.proc = None
        self.lines: list[str] = []
        self._t = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            if self._t:
                self._t.join(timeout=2)

    def summary(self) -> dict:
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
def make_state(w, precision, run_cls, abi, W):
    """Device run primed as the driver primes it: positions on Parker
    spirals, updateMhd, moveNodes, updateMhd, then the seed distribution."""
    g = W.build_grids(w)
    d = w.dims(precision)
    run = run_cls(d, w.params, g)
    nodes = W.initial_nodes(w)
    run.upload_nodes(nodes)
    run.update_mhd(0.0)
    run.move_nodes(w.params.t_del)
    run.update_mhd(w.params.t_del)
    nodes = run.download_nodes()
    return run, g, nodes


def host_f(w, nodes, g, W, pinned=True):
    n = w.cells
    if pinned:
        import torch
        buf = torch.empty(n, dtype=torch.float64, pin_memory=True).numpy()
    else:
        buf = np.empty(n)
    return W.fill_initial_f(w, nodes, g, buf)


def step(run, t, w):
    """One driver step of the hot path (src/eprem.c:620-671)."""
    run.move_nodes(w.params.t_del)
    run.update_mhd(t + w.params.t_del)
    run.update_energetic_particles(t)
    return t + w.params.t_del


def event_pair(stream_ptr):
    import torch
    s = torch.cuda.ExternalStream(stream_ptr)
    return s, torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def flops_of(stats) -> dict:
    return {"stream": FLOPS_PER_CELL_SUBCYCLE["stream"] * stats.stream_cell_subcycles,
            "node": FLOPS_PER_CELL_SUBCYCLE["focus"] * stats.focus_cell_subcycles
            + FLOPS_PER_CELL_SUBCYCLE["change"] * stats.change_cell_subcycles}


def timed_steps(run, w, steps, t0):
    """K steps on device-resident state, CUDA events on the run's stream."""
    import torch
    s, e0, e1 = event_pair(run.stream)
    run.read_stats()
    run.set_kernel_timing(True)
    run.read_kernel_timing()
    n0 = run.kernel_launches
    torch.cuda.synchronize()
    e0.record(s)
    t = t0
    for _ in range(steps):
        t = step(run, t, w)
    e1.record(s)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    launches = run.kernel_launches - n0
    kt = run.read_kernel_timing()
    stats = run.read_stats()
    run.set_kernel_timing(False)
    return ms, launches, kt, stats, t


def roofline(kt, stats, steps, peak_tflops, hbm_peak, cells, form):
    """Roofline of the dominant kernel: algorithmic flops per launch over the
    kernel's mean CUDA-event duration, against the measured FMA peak."""
    kind = max(("stream", "node"), key=lambda k: kt[k][1])
    launches, total_ms = kt[kind]
    fl = flops_of(stats)[kind]
    per_launch_flops = fl / launches
    mean_s = total_ms / launches * 1e-3
    achieved = per_launch_flops / mean_s / 1e12
    # algorithmic HBM bytes: one read + one write of f per operator pass
    bytes_per_launch = cells * BYTES_PER_CELL_UPDATE[form] / 2.0
    return {
        "kernel": ({"fp32": "k_stream2_pairs", "fp64": "k_stream"}[form] if kind == "stream"
                   else {"fp32": "k_focus32+k_change32", "fp64": "k_node"}[form]),
        "bound": "fp64" if form == "fp64" else "fp32",
        "achieved": round(achieved, 3), "peak": round(peak_tflops, 3), "unit": "TFLOP/s",
        "frac": round(achieved / peak_tflops, 4),
        "peak_source": "measured FMA-chain kernel on this GPU (eprem_gpu_alu_peak)",
        "traffic": (NCU_DRAM_BYTES_PER_CELL[(kind, form)] * cells
                    if (kind, form) in NCU_DRAM_BYTES_PER_CELL else None),
        "traffic_unit": "bytes per launch (ncu DRAM read+write, 96-stream capture scaled by cells)",
        "algorithmic_bytes_per_launch": bytes_per_launch,
        "launches": launches, "mean_launch_ms": round(total_ms / launches, 3),
        "hbm_achieved_gbs": round(bytes_per_launch / mean_s / 1e9, 2),
        "hbm_peak_gbs": hbm_peak,
        "hbm_frac": round(bytes_per_launch / mean_s / 1e9 / hbm_peak, 5) if hbm_peak else None,
        "share_of_step": round(total_ms / sum(v[1] for v in kt.values()), 4),
    }


def measured_peaks():
    try:
        with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as fh:
            return json.load(fh)
    except OSError:
        return {}


# ---------------------------------------------------------------------------
def cpu_sample(w, W, abi, nthreads, min_seconds=10.0):
    """The oracle port on the host cores: `nthreads` streams advanced by EP
    sub-steps of the workload's dt (tDel / numEpSteps), repeated until
    `min_seconds` of CPU work have run -- a bounded sample of the workload.
    Returns (cell-updates/s, seconds, streams, sub-steps)."""
    import ctypes as C
    sys.path.insert(0, os.path.join(HERE, "oracle"))
    import oracle as orc  # CPU baseline leg only
    o = orc.Oracle()
    ns = max(1, min(nthreads, w.num_streams))
    rows = cols = 1
    sub = W.with_faces(w, rows, cols)
    d = sub.dims()
    g = W.build_grids(sub)
    nodes = W.initial_nodes(sub)
    o.update_mhd(d, sub.params, nodes, 0.0)
    o.move_nodes(d, sub.params, nodes, sub.params.t_del)
    o.update_mhd(d, sub.params, nodes, sub.params.t_del)
    # repeat the 6 streams until there are ns of them
    reps = (ns + 5) // 6
    S = 6 * reps
    N = sub.num_nodes
    big_nodes = np.tile(nodes.reshape(abi.NODE_NFIELDS, 6, N), (1, reps, 1)).reshape(
        abi.NODE_NFIELDS, S * N)
    f6 = W.initial_f(sub, nodes, g)
    f = np.tile(f6.reshape(6, -1), (reps, 1)).reshape(-1)
    p = abi.Params.from_buffer_copy(bytes(sub.params))
    p.t_del = sub.params.t_del / sub.params.num_ep_steps
    p.num_ep_steps = 1
    dd = abi.Dims(S, N, 1, sub.num_energies, sub.num_mu, abi.EPREM_FP64)
    gs, keep = W.grids_struct(g)
    substeps = 0
    t0 = time.perf_counter()
    while True:
        rc, st, err = o.update_energetic_particles(dd, p, gs, f, big_nodes, nthreads=nthreads,
                                                   streams=(0, ns))
        if rc:
            raise RuntimeError(err)
        substeps += 1
        dt = time.perf_counter() - t0
        if dt >= min_seconds or substeps >= sub.params.num_ep_steps:
            break
    cells = ns * N * sub.num_energies * sub.num_mu * substeps
    return cells / dt, dt, ns, substeps


def reference_arm(args, rank, ws, dist):
    from eprem_gb300 import abi, workloads as W
    if rank != 0:
        return
    w = W.scale_plain() if args.workload == "scale" else W.small_plain()
    nthreads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_sample(w, W, abi, nthreads, min_seconds=2.0)
    vals, secs = [], []
    for _ in range(args.steps):
        v, dt, ns, nsub = cpu_sample(w, W, abi, nthreads, min_seconds=8.0)
        vals.append(v)
        secs.append(dt)
    value = statistics.mean(vals)
    sample = (f"{ns} streams of the {w.name} workload, {nsub} EP sub-steps each "
              f"(dt = tDel/{w.params.num_ep_steps}), one stream per thread, "
              f"{statistics.mean(secs):.1f} s per step")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(secs),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": w.name, "form": "reference CPU algorithm (oracle port), FP64"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
def ours(args, rank, ws, dist):
    import torch
    from eprem_gb300 import EpremRun, abi, workloads as W
    from eprem_gb300.runtime import alu_peak_tflops

    w = W.scale_plain() if args.workload == "scale" else W.small_plain()
    if ws > 1:
        w.seed += rank  # independent ensemble member per rank
    peaks = measured_peaks()
    fp32_peak = alu_peak_tflops(abi.EPREM_FP32)
    fp64_peak = alu_peak_tflops(abi.EPREM_FP64)

    # ---- device-resident FP32 run ---------------------------------------
    run, g, nodes = make_state(w, abi.EPREM_FP32, EpremRun, abi, W)
    f_host = host_f(w, nodes, g, W, pinned=True)
    run.upload_f(f_host)
    run.synchronize()
    t = w.params.t_del
    for _ in range(args.warmup):
        t = step(run, t, w)
    run.synchronize()
    barrier(dist)
    torch.cuda.synchronize()
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        ms, launches, kt, stats, t = timed_steps(run, w, args.steps, t)
    torch.cuda.synchronize()
    barrier(dist)
    ms_max = reduce_max(dist, ms)
    cell_updates = w.cells * w.params.num_ep_steps * args.steps
    value = cell_updates * ws / (ms_max * 1e-3)
    roof = roofline(kt, stats, args.steps, fp32_peak, peaks.get("hbm_gbs"), w.cells, "fp32")

    # ---- end to end through the C ABI with host buffers ------------------
    nodes_host = torch.empty(nodes.size, dtype=torch.float64, pin_memory=True).numpy()
    nodes_host[:] = run.download_nodes().reshape(-1)
    nodes_host = nodes_host.reshape(abi.NODE_NFIELDS, -1)
    f_host[:] = run.download_f(f_host)
    s, e0, e1 = event_pair(run.stream)
    barrier(dist)
    torch.cuda.synchronize()
    e0.record(s)
    for _ in range(args.e2e_steps):
        # the step with every input copied in and every output copied out:
        # node fields around it, f through the pipelined host-buffer update
        run.upload_nodes(nodes_host)
        run.move_nodes(w.params.t_del)
        run.update_mhd(t + w.params.t_del)
        run.update_energetic_particles_host(f_host, f_host, t)
        t += w.params.t_del
        run.download_nodes(nodes_host)
    e1.record(s)
    e1.synchronize()
    e2e_ms = reduce_max(dist, e0.elapsed_time(e1))
    e2e_value = w.cells * w.params.num_ep_steps * args.e2e_steps * ws / (e2e_ms * 1e-3)
    h2d = f_host.nbytes + nodes_host.nbytes
    run.close()
    del f_host

    # ---- plain FP64 form and the FP32 flux error on a stream subset ------
    plain = None
    if not args.skip_fp64 and rank == 0:
        sub = W.with_faces(w, args.fp64_faces, args.fp64_faces)
        r64, g64, n64 = make_state(sub, abi.EPREM_FP64, EpremRun, abi, W)
        r32, _, _ = make_state(sub, abi.EPREM_FP32, EpremRun, abi, W)
        f0 = host_f(sub, n64, g64, W, pinned=False)
        r64.upload_f(f0)
        r32.upload_f(f0)
        tt = sub.params.t_del
        tt = step(r64, tt, sub)
        step(r32, sub.params.t_del, sub)
        r32.synchronize()
        ms64, l64, kt64, st64, _ = timed_steps(r64, sub, 1, tt)
        ms32, _, _, _, _ = timed_steps(r32, sub, 1, tt)
        j64 = r64.omni_flux()
        j32 = r32.omni_flux()
        mask = j64 > 1e-30 * j64.max()
        flux_err = float(np.max(np.abs(j32[mask] - j64[mask]) / j64[mask]))
        cu = sub.cells * sub.params.num_ep_steps
        plain = {
            "value": cu / (ms64 * 1e-3), "unit": UNIT, "streams": sub.num_streams,
            "ms_per_step": ms64,
            "fp32_same_subset_value": cu / (ms32 * 1e-3),
            "roofline": roofline(kt64, st64, 1, fp64_peak, peaks.get("hbm_gbs"), sub.cells,
                                 "fp64"),
            "flux_rel_err_fp32_vs_fp64": flux_err,
            "flux_err_steps": 2,
        }
        if not args.skip_surrogate:
            plain["split_and_surrogate"] = surrogate_case(args, EpremRun, abi, W, j64, sub)
        r64.close()
        r32.close()

    # ---- MHD-coupled (MAS) workload ----------------------------------------
    mas = None
    if not args.skip_mas and rank == 0:
        mas = mas_case(args, EpremRun, abi, W, fp32_peak, peaks.get("hbm_gbs"))

    # ---- batched ensemble --------------------------------------------------
    ensemble = None
    if not args.skip_ensemble and rank == 0:
        from eprem_gb300 import Ensemble
        ensemble = ensemble_case(args, EpremRun, Ensemble, abi, W)

    # ---- CPU baseline ----------------------------------------------------
    cpu = None
    if not args.skip_cpu and rank == 0 and ws == 1:
        nthreads = os.cpu_count() or 1
        v, dt, ns, nsub = cpu_sample(w, W, abi, nthreads, min_seconds=12.0)
        cpu = {"value": v, "unit": UNIT, "cores": nthreads, "kind": "port",
               "sample": f"{ns} streams x {nsub} EP sub-steps of the same workload "
                         f"({dt:.1f} s, one stream per thread)"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {
                "workload": w.name, "form": "FP32 f and stencils, FP64 positions/ds/CFL",
                "streams": w.num_streams, "nodes": w.num_nodes, "energies": w.num_energies,
                "mu": w.num_mu, "ep_substeps_per_step": w.params.num_ep_steps,
                "t_del_s": w.params.t_del * W.TAU, "step": "moveNodes+updateMhd+updateEnergeticParticles",
                "l2": "inputs larger than L2 (f = %.1f GB on the device)" % (w.cells * 4 / 1e9),
                "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU",
            },
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": h2d, "steps": args.e2e_steps},
            "gpu_launches": launches,
            "roofline": roof,
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
            "plain_fp64": plain,
            "mhd_coupled": mas,
            "ensemble": ensemble,
            "alu_peaks_tflops": {"fp32": fp32_peak, "fp64": fp64_peak},
            "stats_last_step": stats.as_dict(),
        }
        print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
class MasSlices:
    """masGetInterpData's role for the bench (src/readMAS.c:645-998): the two
    slices bounding a time are on the device (slot = slice index mod 3, so
    the next slice can be loaded while the current pair stays selected), and
    s_cor interpolates between them."""

    def __init__(self, run, grid, W, t_end):
        self.run, self.grid, self.W = run, grid, W
        self.slot_of = {}
        self.keep = {}
        self.h2d_bytes = 0
        # the synthetic slices are made on the host before any timing, as the
        # reference reads its slice files outside its hot path
        last = int(np.searchsorted(grid.times, t_end, side="right"))
        self.fields = {k: grid.slice_fields(grid.times[k])
                       for k in range(min(last + 1, len(grid.times)))}

    def _load(self, k):
        if k in self.slot_of:
            return self.slot_of[k]
        slot = k % 3
        for kk in [kk for kk, sl in self.slot_of.items() if sl == slot]:
            del self.slot_of[kk]
            self.keep.pop(kk, None)
        fields = self.fields[k]
        st, keep = self.W.mas_slice_struct(self.grid, fields)
        self.run.mas_load_slice(slot, st)
        self.h2d_bytes += sum(a.nbytes for a in fields.values())
        self.keep[k] = (st, keep, fields)
        self.slot_of[k] = slot
        return slot

    def select(self, t):
        times = self.grid.times
        k0 = int(np.searchsorted(times, t, side="right") - 1)
        k0 = min(max(k0, 0), len(times) - 2)
        s_cor = (t - times[k0]) / (times[k0 + 1] - times[k0])
        a, b = self._load(k0), self._load(k0 + 1)
        self.run.mas_select(a, b, float(min(max(s_cor, 0.0), 1.0)), 0.0)


def mas_case(args, EpremRun, abi, W, fp32_peak, hbm_peak):
    """The MHD-coupled workload: 1536 streams x 1500 nodes x 40 E x 40 mu in
    the FP32 form on a synthetic 300 x 180 x 360 staggered MAS grid (1-30 Rs)
    with a CME pulse, 16 slices an hour apart; a step is masMoveNodes (RK4
    through the interpolated V) + masGetInterpData + updateMhd (trilinear
    interpolation of B, V, rho at every node) + updateEnergeticParticles."""
    import torch
    w = W.mas_workload(16, 16, 1500, 40, 40, r_min_au=0.006, r_max_au=1.0,
                       name="mhd-coupled 1536x1500x40x40 on a 300x180x360 MAS grid")
    grid = W.mas_grid(nr=300, nt=180, np_=360, r_min_rs=1.0, r_max_rs=30.0, n_slices=16)
    g = W.build_grids(w)
    run = EpremRun(w.dims(abi.EPREM_FP32), w.params, g)
    nodes = W.initial_nodes(w)
    run.upload_nodes(nodes)
    mp = abi.MasParams.from_buffer_copy(bytes(grid.params))
    mp.max_slices = 3
    run.mas_init(mp)
    td = w.params.t_del
    sl = MasSlices(run, grid, W, td * (args.mas_steps + 4))
    sl.select(0.0)
    run.update_mhd(0.0)
    run.mas_move_nodes(td)
    sl.select(td)
    run.update_mhd(td)
    nodes = run.download_nodes()
    f = W.fill_initial_f(w, nodes, g, np.empty(w.cells))
    run.upload_f(f)
    del f
    run.synchronize()

    def mas_step(t):
        run.mas_move_nodes(td)           # src/eprem.c:621, interpolation data of time t
        sl.select(t + td)                # masGetInterpData(tDel), :638
        run.update_mhd(t + td)           # :639
        run.update_energetic_particles(t)
        return t + td

    t = td
    t = mas_step(t)
    run.synchronize()
    s, e0, e1 = event_pair(run.stream)
    run.read_stats()
    run.set_kernel_timing(True)
    run.read_kernel_timing()
    n0 = run.kernel_launches
    torch.cuda.synchronize()
    h0 = sl.h2d_bytes
    e0.record(s)
    for _ in range(args.mas_steps):
        t = mas_step(t)
    e1.record(s)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    kt = run.read_kernel_timing()
    stats = run.read_stats()
    launches = run.kernel_launches - n0
    run.set_kernel_timing(False)
    out = {
        "value": w.cells * w.params.num_ep_steps * args.mas_steps / (ms * 1e-3),
        "unit": UNIT, "workload": w.name, "steps": args.mas_steps, "warmup": 1,
        "ms_per_step": ms / args.mas_steps, "dtype": "f32",
        "step": "masMoveNodes(RK4)+masGetInterpData+updateMhd(MAS)+updateEnergeticParticles",
        "mas_grid": {"nr": grid.nr, "nt": grid.nt, "np": grid.np_, "slices": len(grid.times),
                     "slice_h2d_bytes_in_timed_steps": sl.h2d_bytes - h0},
        "kernel_ms_per_step": {k: v[1] / args.mas_steps for k, v in kt.items() if v[0]},
        "gpu_launches": launches,
        "roofline": roofline(kt, stats, args.mas_steps, fp32_peak, hbm_peak, w.cells, "fp32"),
    }
    run.close()
    return out


def ensemble_case(args, EpremRun, Ensemble, abi, W):
    """The batched-ensemble workload: the first n of 64 runs with uneven
    sizes and parameters (24-1536 streams, 400-2000 nodes, 20-50 E, 20-40 mu,
    seed index, mean free path and shock speed drawn from a fixed seed) in
    the FP32 form, streaming shapes autotuned per size class, one CUDA-graph
    launch per step for all runs.  Beside it, the same runs from the same
    state stepped one after another through the per-run entry points (each
    run's step completes before the next run's starts): both legs re-create
    the state (nodes, background, seed population), take one untimed step and
    time the same K steps, so both do the same sub-cycles."""
    import torch
    members = W.ensemble_members(64)[: args.ensemble_runs]
    runs = [EpremRun(w.dims(abi.EPREM_FP32), w.params, W.build_grids(w)) for w in members]

    def initial_state():
        for run, w in zip(runs, members):
            run.upload_nodes(W.initial_nodes(w))
            run.update_mhd(0.0)
            run.move_nodes(w.params.t_del)
            run.update_mhd(w.params.t_del)
            run.init_seed_population(w.seed, w.perturb)
        torch.cuda.synchronize()

    cells = sum(w.cells * w.params.num_ep_steps for w in members)
    initial_state()
    t_tune = time.perf_counter()
    ens = Ensemble(runs)
    chosen = ens.autotune()
    t_tune = time.perf_counter() - t_tune
    K = args.ensemble_steps

    # one after another, per-run entry points, host-timed around device syncs
    initial_state()
    seq_s = 0.0
    for k in range(1 + K):
        t0 = time.perf_counter()
        for run, w in zip(runs, members):
            t = (1 + k) * w.params.t_del
            run.move_nodes(w.params.t_del)
            run.update_mhd(t + w.params.t_del)
            run.update_energetic_particles(t)
            run.synchronize()
        if k:
            seq_s += time.perf_counter() - t0

    # the same steps from the same state, one graph launch per step, for two
    # graph schedules: one branch per run side by side, and the runs in one
    # serial chain (the default); `value` is the default's
    by_chains = {}
    for chains in (0, 1):
        initial_state()
        ens.set_chains(chains)
        ens.set_time([w.params.t_del for w in members])
        ens.step()  # capture + the untimed step
        ens.synchronize()
        s, e0, e1 = event_pair(ens.stream)
        n0 = sum(r.kernel_launches for r in runs)
        e0.record(s)
        for _ in range(K):
            ens.step()
        e1.record(s)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        ens.synchronize()
        launches = sum(r.kernel_launches for r in runs) - n0
        by_chains[chains] = cells * K / (ms * 1e-3)
    out = {
        "value": cells * K / (ms * 1e-3), "unit": UNIT,
        "value_by_schedule": {"branch_per_run": by_chains[0], "one_chain": by_chains[1]},
        "runs": len(members), "of_runs": 64, "total_cells": sum(w.cells for w in members),
        "sizes": [w.name.split(": ")[1] for w in members],
        "steps": K, "warmup": 1, "ms_per_step": ms / K,
        "graph_launches_per_step": 1, "kernel_launches_per_step": launches // K,
        "one_by_one_value": cells * K / seq_s,
        "speedup_vs_one_by_one": (cells * K / (ms * 1e-3)) / (cells * K / seq_s),
        "autotuned_stream_variants": chosen, "autotune_s": round(t_tune, 3), "dtype": "f32",
    }
    ens.close()
    for r in runs:
        r.close()
    return out


def surrogate_case(args, EpremRun, abi, W, j64, sub):
    """The learned focusing step and the split form on the 96-stream subset
    of the precision-at-scale workload.  The surrogate is trained on rows of
    ten successive states (the plain focusing of each row as the target), its
    residual tolerance calibrated on them; then one step of each form is
    timed and its flux compared with the FP64 reference form (j64):
      * surrogate_focus: the reference's scheme, focusing by the surrogate
        (rows failing the residual check by the plain kernel);
      * split: relaxation moved from the streaming sub-cycles to one exact
        step after the focusing (plain kernels) -- a change of the operator
        splitting, reported for its error."""
    import torch
    from eprem_gb300.runtime import (NODE_PHASE_SPLIT, NODE_PHASE_SURROGATE_FOCUS, Surrogate,
                                     set_node_phase, surrogate_counts)
    t0 = time.perf_counter()
    src, g, nodes = make_state(sub, abi.EPREM_FP32, EpremRun, abi, W)
    f0 = host_f(sub, nodes, g, W, pinned=False)
    src.upload_f(f0)
    sur = Surrogate(seed=7, chunk_rows=1 << 20)
    sur.reserve(6_000_000)
    n = 0
    t = sub.params.t_del
    for k in range(10):
        n = sur.collect(src, rate=0.1, seed=1000 + k)
        t = step(src, t, sub)
    src.close()
    t_collect = time.perf_counter() - t0
    t0 = time.perf_counter()
    l0 = sur.train(1, 8192, 1e-3)
    l1 = sur.train(args.surrogate_train_steps, 8192, 1e-3)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    tol = sur.calibrate(0.999, 1.5)
    out = {"samples": n, "collect_s": round(t_collect, 2), "train_steps": args.surrogate_train_steps,
           "batch": 8192, "train_s": round(t_train, 2), "loss_first": l0, "loss_last": l1,
           "tolerance": tol}
    # the residual tolerance trades rows kept against accuracy: the 0.999,
    # 0.9 and 0.5 quantiles of the plain rows' residuals
    tols = {}
    for q in (0.9, 0.5):
        tols[q] = sur.calibrate(q, 1.0)
    sweep = []
    for q, tq in sorted(tols.items()):
        sur.set_tolerance(tq)
        r, _, _ = make_state(sub, abi.EPREM_FP32, EpremRun, abi, W)
        r.upload_f(f0)
        set_node_phase(r, NODE_PHASE_SURROGATE_FOCUS, sur)
        tt = step(r, sub.params.t_del, sub)
        step(r, tt, sub)
        j = r.omni_flux()
        mask = j64 > 1e-30 * j64.max()
        kept, fb = surrogate_counts(r)
        sweep.append({"quantile": q, "tolerance": tq, "rows_kept_frac": kept / max(1, kept + fb),
                      "flux_rel_err_vs_fp64_reference_form":
                          float(np.max(np.abs(j[mask] - j64[mask]) / j64[mask]))})
        r.close()
    out["tolerance_sweep"] = sweep
    sur.set_tolerance(tol)
    for label, mode in (("surrogate_focus", NODE_PHASE_SURROGATE_FOCUS), ("split", NODE_PHASE_SPLIT)):
        r, _, _ = make_state(sub, abi.EPREM_FP32, EpremRun, abi, W)
        r.upload_f(f0)
        set_node_phase(r, mode, sur if mode == NODE_PHASE_SURROGATE_FOCUS else None)
        tt = step(r, sub.params.t_del, sub)
        r.synchronize()
        ms, _, kt, _, _ = timed_steps(r, sub, 1, tt)
        j = r.omni_flux()
        mask = j64 > 1e-30 * j64.max()
        cu = sub.cells * sub.params.num_ep_steps
        entry = {"value": cu / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms,
                 "node_phase_ms": kt["node"][1],
                 "flux_rel_err_vs_fp64_reference_form":
                     float(np.max(np.abs(j[mask] - j64[mask]) / j64[mask]))}
        if mode == NODE_PHASE_SURROGATE_FOCUS:
            kept, fb = surrogate_counts(r)
            entry["rows_kept"] = kept
            entry["rows_fallback"] = fb
        out[label] = entry
        r.close()
    sur.close()
    return out


def profile_step(args):
    """One EP sub-step of the 96-stream subset of the precision-at-scale
    workload (f = 0.77 GB in FP32, above L2): the small case of the ncu
    captures."""
    from eprem_gb300 import EpremRun, abi, workloads as W
    w = W.scale_plain()
    sub = W.with_faces(w, 4, 4)
    sub.params.t_del = w.params.t_del / w.params.num_ep_steps
    sub.params.num_ep_steps = 1
    sub.params.stream_variant = args.stream_variant
    prec = abi.EPREM_FP32 if args.profile_step == "fp32" else abi.EPREM_FP64
    run, g, nodes = make_state(sub, prec, EpremRun, abi, W)
    run.upload_f(W.fill_initial_f(sub, nodes, g, np.empty(sub.cells)))
    extra = {}
    if args.shell_diffusion is not None:
        S, C = sub.num_streams, 4 * sub.cols
        s = np.arange(S)
        run.set_shell_diffusion(np.stack([(s - C) % S, (s + 1) % S, (s - 1) % S, (s + C) % S],
                                         axis=1), args.shell_diffusion)
        run.update_energetic_particles(0.0)
        run.read_stats()
        run.set_kernel_timing(True)
        run.read_kernel_timing()
    run.update_energetic_particles(0.0)
    run.synchronize()
    if args.shell_diffusion is not None:
        extra["kernel_ms"] = {k: v[1] for k, v in run.read_kernel_timing().items() if v[0]}
        extra["shell_diffusion"] = args.shell_diffusion
    print(json.dumps({"profile_step": args.profile_step, "workload": sub.name,
                      "stats": run.read_stats().as_dict(), **extra}))
    run.close()


def main():
    args = parse()
    if args.profile_step:
        profile_step(args)
        return
    if args.ensemble_only:
        from eprem_gb300 import Ensemble, EpremRun, abi, workloads as W
        out = ensemble_case(args, EpremRun, Ensemble, abi, W)
        print(json.dumps({"metric": METRIC, "unit": UNIT, "ensemble": out}), flush=True)
        return
    rank, ws, dist = dist_setup()
    try:
        if args.impl == "reference":
            reference_arm(args, rank, ws, dist)
        else:
            ours(args, rank, ws, dist)
    finally:
        if dist is not None:
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
