"""The oracle's MAS restatement (updateMhd's MHD_MAS branch with masGetNode /
masTriLinear / masWind, and masMoveNodes' RK4) against the reference's own C,
live, on a synthetic staggered MAS grid with a CME pulse.  Nodes cross the
MAS outer radius so both the trilinear path and the Parker extrapolation run.
Needs oracle/_ref (reference tree present); bit equality required."""
import multiprocessing as mp
import os

import numpy as np
import pytest

import oracle as O
from eprem_gb300 import abi, workloads as W

pytestmark = pytest.mark.skipif(not os.path.exists(O.REF_LIB),
                                reason="reference harness not built here")


def _setup():
    w = W.mas_workload(1, 1, 40, 8, 6, r_min_au=0.006, r_max_au=0.5)
    grid = W.mas_grid(nr=24, nt=16, np_=32, n_slices=2, r_max_rs=20.0)
    f0 = grid.slice_fields(grid.times[0] + 0.3 * (grid.times[1] - grid.times[0]))
    f1 = grid.slice_fields(grid.times[1])
    return w, grid, f0, f1


def _reference(q):
    w, grid, f0, f1 = _setup()
    ref = O.Reference()
    ref.setup(w)
    s0, k0 = W.mas_slice_struct(grid, f0)
    s1, k1 = W.mas_slice_struct(grid, f1)
    nodes = W.initial_nodes(w)
    ref.load(np.zeros(w.cells), nodes)
    ref.mas_setup(grid.params, s0, s1, 0.37, 0.21)
    out = []
    ref.update_mhd(0.0)
    for _ in range(2):
        ref.mas_move_nodes(w.params.t_del)
        ref.update_mhd(w.params.t_del)
        n = np.zeros_like(nodes)
        ref.store(np.zeros(w.cells), n)
        out.append(n)
    q.put(out)


def test_mas_update_and_rk4_bit_exact(oracle_lib):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    p = ctx.Process(target=_reference, args=(q,))
    p.start()
    ref_out = q.get(timeout=300)
    p.join()
    w, grid, f0, f1 = _setup()
    s0, k0 = W.mas_slice_struct(grid, f0)
    s1, k1 = W.mas_slice_struct(grid, f1)
    mas = O.MasState(O.C.pointer(s0), O.C.pointer(s1), 0.37, 0.21, grid.params)
    d = w.dims()
    nodes = W.initial_nodes(w)
    oracle_lib.mas_update_mhd(d, w.params, nodes, mas)
    r_au = nodes[abi.NODE["RMAG"]] * w.params.r_scale
    inside = r_au <= grid.params.radial_max * W.RSAU
    assert inside.any() and (~inside).any()  # both branches of masGetNode
    for i in range(2):
        oracle_lib.mas_move_nodes(d, w.params, nodes, mas, w.params.t_del)
        oracle_lib.mas_update_mhd(d, w.params, nodes, mas, w.params.t_del)
        np.testing.assert_array_equal(nodes, ref_out[i])
