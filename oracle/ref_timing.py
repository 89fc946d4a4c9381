"""The CPU baseline: the reference's own updateEnergeticParticles, compiled
with its own flags (oracle/_ref/native/libeprem_ref_native.so, -O3
-march=native), timed on the host's cores -- TEST AND MEASUREMENT
INFRASTRUCTURE ONLY (bench.py's CPU legs call it; nothing on the GPU path
does).

The reference allocates its globals once per process and runs one rank's
streams serially (src/energeticParticles.c:108-174), so the baseline is one
process per core, each holding its own cube-sphere grid of one face-cell per
face (6 streams) with the workload's per-stream sizes (nodes, energies, mu)
and geometry rule: with shell diffusion and drift off every stream is
independent, so P such processes do the work of 6P streams of the full grid.

A sample is a bounded number of EP sub-steps.  The reference derives its
sub-step from tDel / numEpSteps and divides the node's per-step MHD changes
(mhdDuPar, mhdDlnB, mhdDlnN) by dt * numEpSteps; the sample sets
numEpSteps = 1 with tDel / numEpSteps as the step and those three node fields
divided by numEpSteps, so every sub-step does exactly the work (sub-cycle
counts, coefficients) of a sub-step of the full call.
"""
from __future__ import annotations

import dataclasses
import multiprocessing as mp
import os
import time

import numpy as np


def _worker(args):
    workload_name, min_seconds, max_substeps, barrier = args
    import oracle as orc
    from eprem_gb300 import abi, workloads as W
    base = W.scale_plain() if workload_name == "scale" else W.small_plain()
    w = W.with_faces(base, 1, 1)
    o = orc.Oracle()  # the restatement primes the state (bit-equal to the reference)
    d = w.dims()
    g = W.build_grids(w)
    nodes = W.initial_nodes(w)
    o.update_mhd(d, w.params, nodes, 0.0)
    o.move_nodes(d, w.params, nodes, w.params.t_del)
    o.update_mhd(d, w.params, nodes, w.params.t_del)
    f = W.initial_f(w, nodes, g)
    n = w.params.num_ep_steps
    for fld in ("DUPAR", "DLNB", "DLNN"):
        nodes[abi.NODE[fld]] /= n
    p = abi.Params.from_buffer_copy(bytes(w.params))
    p.t_del = w.params.t_del / n
    p.num_ep_steps = 1
    ref = orc.Reference(orc.NATIVE_LIB)
    ref.setup(dataclasses.replace(w, params=p))
    ref.load(f, nodes)
    barrier.wait()
    t0 = time.perf_counter()
    k = 0
    while True:
        rc, _ = ref.update_energetic_particles(0.0)
        if rc:
            raise RuntimeError(f"reference update failed: {rc}")
        k += 1
        dt = time.perf_counter() - t0
        if dt >= min_seconds or k >= max_substeps:
            break
    return w.cells * k, dt, k, w.num_streams


def sample(workload_name: str, processes: int | None = None, min_seconds: float = 8.0,
           max_substeps: int = 30) -> dict:
    """One timed sample: every process runs EP sub-steps of its 6 streams
    until min_seconds have passed (at least one).  Returns the aggregate
    cell-updates/s (all processes' cell-updates over the slowest process's
    time) and what was run."""
    import oracle as orc
    if not os.path.exists(orc.NATIVE_LIB):
        raise RuntimeError("the reference's own build is missing (oracle/Makefile ref-native)")
    P = processes or os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        barrier = m.Barrier(P)
        with ctx.Pool(P) as pool:
            res = pool.map(_worker, [(workload_name, min_seconds, max_substeps, barrier)] * P)
    cells = sum(r[0] for r in res)
    secs = max(r[1] for r in res)
    subs = [r[2] for r in res]
    return {"value": cells / secs, "seconds": secs, "processes": P,
            "streams": sum(r[3] for r in res), "substeps_min": min(subs),
            "substeps_max": max(subs)}


def cpu_model() -> str:
    """The host CPU's model name (lscpu, or /proc/cpuinfo)."""
    import subprocess
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.startswith("Model name:"):
                return ln.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for ln in open("/proc/cpuinfo"):
            if ln.lower().startswith(("model name", "cpu part")):
                return ln.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


if __name__ == "__main__":
    import json
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    print(json.dumps(sample(sys.argv[1] if len(sys.argv) > 1 else "scale",
                            min_seconds=float(sys.argv[2]) if len(sys.argv) > 2 else 4.0)))
