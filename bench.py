"""Benchmark of the GB300 energetic-particle update.

Metric: cell-updates/s, one cell-update = one (node, energy, mu) cell through
one EP sub-step (streaming + isotropisation, focusing, adiabatic change).  A
step is one driver step of the hot path: moveNodes + updateMhd +
updateEnergeticParticles (numEpSteps = 30 sub-steps), src/eprem.c:620-671.

Workload (default): the precision-at-scale case -- 1536 streams x 1000 nodes x
50 energies (0.1-1000 MeV) x 40 mu, Parker wind, seed power law -- in the
chosen form (f and stencil arithmetic in FP32 with a binary exponent per
row, geometry / CFL in FP64).  The plain FP64 form is measured beside it on
48 streams sampled from the 1536, stepped from the same state through the
same steps, and the FP32 omnidirectional flux is compared with it.  Further
legs: the MHD-coupled (MAS) workload, the batched ensembles (8 runs of
uneven sizes; 64 runs of the CPU-runnable case's size), the split form and
the surrogate, and the CPU baseline -- the reference's own C of the path,
built with its own flags, one process per host core.

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
# one ncu capture of the 96-stream subset (profiles/k_stream2_mirror_fp32_96streams.txt,
# profiles/k_stream_fp64_96streams.txt, profiles/k_focus32_k_change32_fp32_96streams.txt):
# traffic per launch / 96*1000*50*40 cells; traffic grows with the number of
# (stream, energy) slabs, so it scales to a full launch by the cells processed.
NCU_DRAM_BYTES_PER_CELL = {("stream", "fp32"): 1603.9058e6 / 192e6,
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
    ap.add_argument("--fp64-streams", type=int, default=48,
                    help="streams of the headline grid (every S/n-th) run in the plain FP64 "
                         "form beside the FP32 run: its timing, and the FP32 flux error")
    ap.add_argument("--mas-fp64-streams", type=int, default=24,
                    help="streams of the MHD-coupled grid run in FP64 for its flux error")
    ap.add_argument("--skip-fp64", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-mas", action="store_true")
    ap.add_argument("--skip-ensemble", action="store_true")
    ap.add_argument("--ensemble-runs", type=int, default=8,
                    help="members of the 64-run batched ensemble to step (first n)")
    ap.add_argument("--ensemble-steps", type=int, default=2)
    ap.add_argument("--ensemble-only", action="store_true",
                    help="measure only the batched ensemble (with --ensemble-runs 64: the full set)")
    ap.add_argument("--skip-ensemble-small", action="store_true")
    ap.add_argument("--ensemble-small-runs", type=int, default=64,
                    help="runs of the CPU-runnable case's size in the small-run ensemble")
    ap.add_argument("--skip-surrogate", action="store_true")
    ap.add_argument("--surrogate-faces", type=int, default=4,
                    help="rows=cols of the surrogate case's grid (6*n*n streams)")
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


def sampled_streams(S, n):
    """n streams spread over the grid (every S/n-th)."""
    return np.arange(0, S, max(1, S // max(1, n)))[:n]


def stream_subset(w, idx, nodes, f, abi):
    """Nodes and f of streams idx of a run of workload w.  Streams are
    independent on this path (no shell diffusion, no drift), so a run of
    these streams alone steps them exactly as the whole run does."""
    S, N = w.num_streams, w.num_nodes
    ns = np.ascontiguousarray(nodes.reshape(abi.NODE_NFIELDS, S, N)[:, idx, :]).reshape(
        abi.NODE_NFIELDS, -1)
    fs = np.ascontiguousarray(f.reshape(S, -1)[idx]).reshape(-1)
    return ns, fs


def flux_rel_err(j, jref):
    """Max relative omnidirectional-flux error over (node, E) with J > 1e-30 max J."""
    mask = jref > 1e-30 * jref.max()
    return float(np.max(np.abs(j[mask] - jref[mask]) / jref[mask]))


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


def roofline(kt, stats, steps, peak_tflops, hbm_peak, cells, form, stream_kernel=None):
    """Roofline of the dominant kernel: algorithmic flops per launch over the
    kernel's mean CUDA-event duration, against the measured FMA peak.
    stream_kernel: the run's streaming kernel (EpremRun.stream_kernel)."""
    kind = max(("stream", "node"), key=lambda k: kt[k][1])
    launches, total_ms = kt[kind]
    fl = flops_of(stats)[kind]
    per_launch_flops = fl / launches
    mean_s = total_ms / launches * 1e-3
    achieved = per_launch_flops / mean_s / 1e12
    # algorithmic HBM bytes: one read + one write of f per operator pass
    bytes_per_launch = cells * BYTES_PER_CELL_UPDATE[form] / 2.0
    return {
        "kernel": ((stream_kernel or {"fp32": "k_stream2", "fp64": "k_stream"}[form])
                   if kind == "stream"
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
    # one sub-step per call with the full call's sub-step work: dt = tDel /
    # numEpSteps, and the per-step MHD changes divided alike (the reference
    # divides them by dt * numEpSteps)
    p = abi.Params.from_buffer_copy(bytes(sub.params))
    p.t_del = sub.params.t_del / sub.params.num_ep_steps
    p.num_ep_steps = 1
    for fld in ("DUPAR", "DLNB", "DLNN"):
        big_nodes[abi.NODE[fld]] /= sub.params.num_ep_steps
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


def cpu_baseline(w, W, abi, min_seconds):
    """One bounded sample of the workload on the host's cores: the
    reference's own C built with its own flags (oracle/_ref/native, one
    process per core, 6 streams each), else -- where the reference tree was
    not there to build it -- the oracle port (one stream per thread)."""
    sys.path.insert(0, os.path.join(HERE, "oracle"))
    import oracle as orc  # CPU baseline leg only
    import ref_timing
    name = "scale" if w.num_streams > 24 else "small"
    if os.path.exists(orc.NATIVE_LIB):
        r = ref_timing.sample(name, min_seconds=min_seconds)
        return {"value": r["value"], "unit": UNIT, "cores": r["processes"], "kind": "reference",
                "cpu_model": ref_timing.cpu_model(), "seconds": r["seconds"],
                "sample": (f"the reference's own updateEnergeticParticles (-O3 "
                           f"{'-mcpu' if os.uname().machine in ('aarch64', 'arm64') else '-march'}"
                           f"=native), {r['processes']} processes x 6 streams of the "
                           f"{w.name} per-stream workload ({r['streams']} streams), "
                           f"{r['substeps_min']}-{r['substeps_max']} EP sub-steps each "
                           f"(dt = tDel/{w.params.num_ep_steps}, the full call's sub-step work), "
                           f"{r['seconds']:.1f} s")}
    nthreads = os.cpu_count() or 1
    v, dt, ns, nsub = cpu_sample(w, W, abi, nthreads, min_seconds=min_seconds)
    return {"value": v, "unit": UNIT, "cores": nthreads, "kind": "port", "seconds": dt,
            "sample": f"oracle port: {ns} streams of {w.name} x {nsub} EP sub-steps "
                      f"({dt:.1f} s, one stream per thread; the reference's own build absent)"}


def reference_arm(args, rank, ws, dist):
    from eprem_gb300 import abi, workloads as W
    if rank != 0:
        return
    w = W.scale_plain() if args.workload == "scale" else W.small_plain()
    for _ in range(args.warmup):
        cpu_baseline(w, W, abi, min_seconds=1.0)
    runs = [cpu_baseline(w, W, abi, min_seconds=6.0) for _ in range(args.steps)]
    value = statistics.mean(r["value"] for r in runs)
    secs = [r["seconds"] for r in runs]
    cb = dict(runs[-1])
    cb["value"] = value
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(secs),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": w.name,
                   "form": "the reference's own C, FP64, on the host cores" if cb["kind"] ==
                   "reference" else "the reference algorithm's CPU restatement, FP64"},
        "cpu_baseline": cb,
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
    # the streams the FP64 form runs beside it, at their initial state
    idx = sampled_streams(w.num_streams, args.fp64_streams)
    nodes_s, f_s = stream_subset(w, idx, nodes, f_host, abi)
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
    # the FP32 flux of the whole run after the timed steps, at the sampled streams
    steps_done = args.warmup + args.steps
    j32_s = run.omni_flux().reshape(w.num_streams, -1)[idx].reshape(-1)
    cell_updates = w.cells * w.params.num_ep_steps * args.steps
    value = cell_updates * ws / (ms_max * 1e-3)
    roof = roofline(kt, stats, args.steps, fp32_peak, peaks.get("hbm_gbs"), w.cells, "fp32",
                    run.stream_kernel)

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

    # ---- plain FP64 form on sampled streams, and the FP32 flux error -------
    # The sampled streams run in FP64 from the same initial state through the
    # same steps as the FP32 run (warm-up + timed); the FP32 flux of the whole
    # run after its timed steps is compared with theirs.  The FP64 form's
    # timing and roofline are its last step.
    plain = None
    if not args.skip_fp64 and rank == 0:
        sub = W.with_faces(w, 1, 1)
        n = len(idx)
        d64 = abi.Dims(n, w.num_nodes, 1, w.num_energies, w.num_mu, abi.EPREM_FP64)
        r64 = EpremRun(d64, w.params, g)
        r64.upload_nodes(nodes_s)
        r64.upload_f(f_s)
        tt = w.params.t_del
        for _ in range(steps_done - 1):
            tt = step(r64, tt, w)
        ms64, l64, kt64, st64, _ = timed_steps(r64, w, 1, tt)
        k64 = r64.stream_kernel
        j64 = r64.omni_flux()
        flux_err = flux_rel_err(j32_s, j64)
        d32 = abi.Dims(n, w.num_nodes, 1, w.num_energies, w.num_mu, abi.EPREM_FP32)
        r32 = EpremRun(d32, w.params, g)
        r32.upload_nodes(nodes_s)
        r32.upload_f(f_s)
        tt = step(r32, w.params.t_del, w)
        ms32, _, _, _, _ = timed_steps(r32, w, 1, tt)
        r32.close()
        cells_s = n * w.num_nodes * w.num_energies * w.num_mu
        cu = cells_s * w.params.num_ep_steps
        plain = {
            "value": cu / (ms64 * 1e-3), "unit": UNIT, "streams": n,
            "streams_sampled": f"every {w.num_streams // n}th of the {w.num_streams}",
            "ms_per_step": ms64,
            "fp32_same_streams_value": cu / (ms32 * 1e-3),
            "roofline": roofline(kt64, st64, 1, fp64_peak, peaks.get("hbm_gbs"), cells_s,
                                 "fp64", k64),
            "flux_rel_err_fp32_vs_fp64": flux_err,
            "flux_err_of": (f"the headline FP32 run after its {steps_done} steps (warm-up + "
                            f"timed), at {n} sampled streams, against the FP64 form's run of "
                            f"those streams through the same steps; J > 1e-30 max J"),
        }
        if not args.skip_surrogate:
            plain["split_and_surrogate"] = surrogate_case(
                args, EpremRun, abi, W, None, W.with_faces(w, args.surrogate_faces,
                                                           args.surrogate_faces))
        r64.close()

    # ---- MHD-coupled (MAS) workload ----------------------------------------
    mas = None
    if not args.skip_mas and rank == 0:
        mas = mas_case(args, EpremRun, abi, W, fp32_peak, peaks.get("hbm_gbs"))

    # ---- batched ensemble --------------------------------------------------
    ensemble = None
    if not args.skip_ensemble and rank == 0:
        from eprem_gb300 import Ensemble
        ensemble = ensemble_case(args, EpremRun, Ensemble, abi, W)
    ensemble_small = None
    if not args.skip_ensemble_small and rank == 0:
        from eprem_gb300 import Ensemble
        ensemble_small = ensemble_case(
            args, EpremRun, Ensemble, abi, W,
            members=W.ensemble_members_small(args.ensemble_small_runs), steps=4,
            schedules=(-1,),
            what="a parameter sweep of runs of the CPU-runnable case's size")

    # ---- CPU baseline ----------------------------------------------------
    cpu = None
    if not args.skip_cpu and rank == 0 and ws == 1:
        cpu = cpu_baseline(w, W, abi, min_seconds=10.0)
        if plain:
            plain["vs_cpu_fp64"] = {
                "fp64_gpu": plain["value"], "fp64_cpu": cpu["value"], "cpu_kind": cpu["kind"],
                "ratio": plain["value"] / cpu["value"]}

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
            "ensemble_small": ensemble_small,
            "alu_peaks_tflops": {"fp32": fp32_peak, "fp64": fp64_peak},
            "stats_last_step": stats.as_dict(),
        }
        print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
class MasSlices:
    """masGetInterpData's role for the bench (src/readMAS.c:645-998): the two
    slices bounding a time are on the device (slot = slice index mod 3) and
    s_cor interpolates between them; prefetch queues the slice after the pair
    on the run's copy stream (eprem_gpu_mas_load_slice_async, from
    page-locked host memory) while the current pair is in use, so a step
    that moves to the next pair finds its slice already loaded."""

    def __init__(self, run, grid, W, t_end, pinned=False):
        self.run, self.grid, self.W = run, grid, W
        self.slot_of = {}
        self.keep = {}
        self.h2d_bytes = 0        # copied synchronously (select found the slice missing)
        self.h2d_async_bytes = 0  # queued on the copy stream ahead of use
        self.pins = []
        # the synthetic slices are made on the host before any timing, as the
        # reference reads its slice files outside its hot path
        last = int(np.searchsorted(grid.times, t_end, side="right"))
        self.fields = {k: grid.slice_fields(grid.times[k])
                       for k in range(min(last + 2, len(grid.times)))}
        if pinned:
            import torch
            for fl in self.fields.values():
                for name, a in fl.items():
                    t = torch.empty(a.shape, dtype=torch.float32, pin_memory=True)
                    tn = t.numpy()
                    tn[...] = a
                    fl[name] = tn
                    self.pins.append(t)

    def _evict(self, slot):
        for kk in [kk for kk, sl in self.slot_of.items() if sl == slot]:
            del self.slot_of[kk]
            self.keep.pop(kk, None)

    def _load(self, k):
        if k in self.slot_of:
            return self.slot_of[k]
        slot = k % 3
        self._evict(slot)
        fields = self.fields[k]
        st, keep = self.W.mas_slice_struct(self.grid, fields)
        self.run.mas_load_slice(slot, st)
        self.h2d_bytes += sum(a.nbytes for a in fields.values())
        self.keep[k] = (st, keep, fields)
        self.slot_of[k] = slot
        return slot

    def _pair(self, t):
        times = self.grid.times
        k0 = int(np.searchsorted(times, t, side="right") - 1)
        return min(max(k0, 0), len(times) - 2)

    def select(self, t):
        times = self.grid.times
        k0 = self._pair(t)
        s_cor = (t - times[k0]) / (times[k0 + 1] - times[k0])
        a, b = self._load(k0), self._load(k0 + 1)
        self.selected = (k0, k0 + 1)
        self.run.mas_select(a, b, float(min(max(s_cor, 0.0), 1.0)), 0.0)

    def prefetch(self):
        """Queue the slice after the selected pair into the third slot."""
        k = self.selected[1] + 1
        if k >= len(self.fields) or k in self.slot_of:
            return
        slot = k % 3
        self._evict(slot)
        fields = self.fields[k]
        st, keep = self.W.mas_slice_struct(self.grid, fields)
        self.run.mas_load_slice_async(slot, st)
        self.h2d_async_bytes += sum(a.nbytes for a in fields.values())
        self.keep[k] = (st, keep, fields)
        self.slot_of[k] = slot


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
    sl = MasSlices(run, grid, W, td * (args.mas_steps + 4), pinned=True)
    sl.select(0.0)
    # the analytic wind first: beyond the MAS radius masWind extrapolates
    # from a node's own fields (src/masInterp.c:1007-1065), which the
    # reference's nodes carry from their way out through the MAS domain
    run.mas_use(False)
    run.update_mhd(0.0)
    run.mas_use(True)
    run.update_mhd(0.0)
    run.mas_move_nodes(td)
    sl.select(td)
    run.update_mhd(td)
    nodes = run.download_nodes()
    f = W.fill_initial_f(w, nodes, g, np.empty(w.cells))
    run.upload_f(f)
    idx = sampled_streams(w.num_streams, args.mas_fp64_streams)
    nodes_s, f_s = stream_subset(w, idx, nodes, f, abi)  # FP64 comparison run's start
    del f
    run.synchronize()

    def mas_step(t):
        run.mas_move_nodes(td)           # src/eprem.c:621, interpolation data of time t
        sl.select(t + td)                # masGetInterpData(tDel), :638
        run.update_mhd(t + td)           # :639
        run.update_energetic_particles(t)
        sl.prefetch()                    # the next slice, copied while this step computes
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
    h0, a0 = sl.h2d_bytes, sl.h2d_async_bytes
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
    j32_s = run.omni_flux().reshape(w.num_streams, -1)[idx].reshape(-1)
    steps_done = 1 + args.mas_steps
    # the sampled streams in FP64 from the same state, background and slices
    r64 = EpremRun(abi.Dims(len(idx), w.num_nodes, 1, w.num_energies, w.num_mu,
                            abi.EPREM_FP64), w.params, g)
    r64.upload_nodes(nodes_s)
    r64.upload_f(f_s)
    r64.mas_init(mp)
    sl64 = MasSlices(r64, grid, W, td * (args.mas_steps + 4))
    sl64.select(td)
    tt = td
    for _ in range(steps_done):
        r64.mas_move_nodes(td)
        sl64.select(tt + td)
        r64.update_mhd(tt + td)
        r64.update_energetic_particles(tt)
        tt += td
    j64 = r64.omni_flux()
    r64.close()
    del sl64
    out = {
        "flux_rel_err_fp32_vs_fp64": flux_rel_err(j32_s, j64),
        "flux_err_of": (f"the FP32 run after its {steps_done} steps, at {len(idx)} sampled "
                        f"streams, against the FP64 form's run of those streams through the "
                        f"same steps and MAS slices; J > 1e-30 max J"),
        "value": w.cells * w.params.num_ep_steps * args.mas_steps / (ms * 1e-3),
        "unit": UNIT, "workload": w.name, "steps": args.mas_steps, "warmup": 1,
        "ms_per_step": ms / args.mas_steps, "dtype": "f32",
        "step": "masMoveNodes(RK4)+masGetInterpData+updateMhd(MAS)+updateEnergeticParticles",
        "mas_grid": {"nr": grid.nr, "nt": grid.nt, "np": grid.np_, "slices": len(grid.times),
                     "slice_h2d_bytes_in_timed_steps_synchronous": sl.h2d_bytes - h0,
                     "slice_h2d_bytes_in_timed_steps_on_copy_stream":
                         sl.h2d_async_bytes - a0},
        "kernel_ms_per_step": {k: v[1] / args.mas_steps for k, v in kt.items() if v[0]},
        "gpu_launches": launches,
        "roofline": roofline(kt, stats, args.mas_steps, fp32_peak, hbm_peak, w.cells, "fp32",
                             run.stream_kernel),
    }
    run.close()
    return out


def ensemble_case(args, EpremRun, Ensemble, abi, W, members=None, steps=None,
                  schedules=(0, 1, -1), what=None):
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
    if members is None:
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
    K = steps or args.ensemble_steps

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
    # graph schedules: one branch per run side by side, the runs in one
    # serial chain, and lock-step with merged streaming launches (the
    # default, last); `value` is the default's
    by_chains = {}
    for chains in schedules:
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
    # FP32 flux error of the smallest stepped member, after the 1 + K steps of
    # the last leg, against its FP64 run from the same state
    im = min(range(len(members)), key=lambda i: members[i].cells)
    wm = members[im]
    j32 = runs[im].omni_flux()
    r64 = EpremRun(wm.dims(abi.EPREM_FP64), wm.params, W.build_grids(wm))
    r64.upload_nodes(W.initial_nodes(wm))
    r64.update_mhd(0.0)
    r64.move_nodes(wm.params.t_del)
    r64.update_mhd(wm.params.t_del)
    r64.init_seed_population(wm.seed, wm.perturb)
    tt = wm.params.t_del
    for _ in range(1 + K):
        tt = step(r64, tt, wm)
    ens_err = flux_rel_err(j32, r64.omni_flux())
    r64.close()
    out = {
        "workload": what or "the first runs of the 64-run ensemble of uneven sizes",
        "flux_rel_err_fp32_vs_fp64": ens_err,
        "flux_err_of": (f"member {im} ({wm.name.split(': ')[1]}, the smallest stepped) after "
                        f"{1 + K} graph steps, against its FP64 run from the same state; "
                        f"J > 1e-30 max J"),
        "value": cells * K / (ms * 1e-3), "unit": UNIT,
        "value_by_schedule": {{0: "branch_per_run", 1: "one_chain",
                               -1: "lockstep_merged_streaming"}[c]: v
                              for c, v in by_chains.items()},
        "runs": len(members), "of_runs": 64 if what is None else len(members),
        "total_cells": sum(w.cells for w in members),
        "sizes": (sorted(set(w.name.split(": ")[1] for w in members)) if what else
                  [w.name.split(": ")[1] for w in members]),
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
    if j64 is None:  # the FP64 reference form's flux after the two compared steps
        r64, _, _ = make_state(sub, abi.EPREM_FP64, EpremRun, abi, W)
        r64.upload_f(f0)
        step(r64, step(r64, sub.params.t_del, sub), sub)
        j64 = r64.omni_flux()
        r64.close()
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
    out = {"samples": n, "collect_s": round(t_collect, 2), "train_steps": args.surrogate_train_steps,
           "batch": 8192, "train_s": round(t_train, 2), "loss_first": l0, "loss_last": l1}
    # the residual check's tolerance from the rows' true distance to their
    # plain step (collected rows): the largest residual below which every
    # calibration row is within the target -- the rows kept at each target,
    # and the flux error of two steps with the surrogate at that tolerance
    sweep = []
    for target in (1e-3, 1e-2, 1e-1):
        tq, kept_cal, within = sur.calibrate_error(target, 1 << 20)
        sur.set_tolerance(tq)
        r, _, _ = make_state(sub, abi.EPREM_FP32, EpremRun, abi, W)
        r.upload_f(f0)
        set_node_phase(r, NODE_PHASE_SURROGATE_FOCUS, sur)
        tt = step(r, sub.params.t_del, sub)
        step(r, tt, sub)
        j = r.omni_flux()
        kept, fb = surrogate_counts(r)
        sweep.append({"row_target": target, "tolerance": tq,
                      "calibration_rows_kept_frac": kept_cal,
                      "calibration_rows_within_target_frac": within,
                      "rows_kept_frac": kept / max(1, kept + fb),
                      "flux_rel_err_vs_fp64_reference_form": flux_rel_err(j, j64)})
        r.close()
    out["tolerance_sweep"] = sweep
    tol, _, _ = sur.calibrate_error(1e-3, 1 << 20)
    out["tolerance"] = tol
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
