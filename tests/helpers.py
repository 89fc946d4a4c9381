"""Shared helpers of the test suite: build a primed run state and run the
oracle or the GPU on it."""
import numpy as np

from eprem_gb300 import abi, workloads as W


def primed_state(w, orc, precision=abi.EPREM_FP64):
    """Positions on Parker spirals, analytic MHD after one node push
    (updateMhd, moveNodes, updateMhd as the driver does, src/eprem.c:620-639),
    and the perturbed seed distribution."""
    d = w.dims(precision)
    g = W.build_grids(w)
    nodes = W.initial_nodes(w)
    orc.update_mhd(d, w.params, nodes, 0.0)
    orc.move_nodes(d, w.params, nodes, w.params.t_del)
    orc.update_mhd(d, w.params, nodes, w.params.t_del)
    f = W.initial_f(w, nodes, g)
    return d, g, f, nodes


def oracle_update(orc, w, g, f, nodes, calls=1, nthreads=8):
    f = f.copy()
    nodes = nodes.copy()
    gs, keep = W.grids_struct(g)
    stats = []
    for _ in range(calls):
        rc, st, err = orc.update_energetic_particles(w.dims(), w.params, gs, f, nodes,
                                                     nthreads=nthreads)
        assert rc == 0, err
        stats.append(st)
    return f, nodes, stats


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b) / np.abs(b)))
