"""MAS background on the GPU (masGetNode trilinear interpolation + masWind
beyond the MAS outer radius, src/masInterp.c:31-68 and src/flow.c:36-154; the
RK4 node push masMoveNodes, src/masInterp.c:1344-1393) against the oracle's
restatement, which is pinned bit-exact to the reference.  Both sides compute
in FP64 from the same float meshes; the GPU may contract multiply-adds, so
fields agree to a relative 1e-10 of each field's scale rather than bitwise."""
import numpy as np
import pytest

import oracle as O
from eprem_gb300 import EpremRun, abi, workloads as W

pytestmark = pytest.mark.gpu

FIELDS_CHECKED = [n for n in abi.NODE_FIELDS
                  if n not in ("DS", "BMAG_PLUS", "BMAG_MINUS")]


def _case(rows=1, cols=1, nodes=40):
    w = W.mas_workload(rows, cols, nodes, 8, 6, r_min_au=0.006, r_max_au=0.5)
    grid = W.mas_grid(nr=24, nt=16, np_=32, n_slices=3, r_max_rs=20.0)
    f0 = grid.slice_fields(grid.times[0] + 0.3 * (grid.times[1] - grid.times[0]))
    f1 = grid.slice_fields(grid.times[1])
    return w, grid, f0, f1


def _assert_nodes_close(a, b, what):
    for name in FIELDS_CHECKED:
        i = abi.NODE[name]
        # a first update from zeroed "old" fields gives infinite and NaN
        # derivatives on both sides; they must sit in the same places
        same = (a[i] == b[i]) | (np.isnan(a[i]) & np.isnan(b[i]))
        assert np.array_equal(np.isfinite(a[i]), np.isfinite(b[i])), f"{what}: field {name}"
        fin = np.isfinite(b[i])
        scale = max(np.max(np.abs(b[i][fin]), initial=0.0), 1e-300)
        diff = np.where(same, 0.0, np.abs(a[i] - b[i]))
        err = np.max(diff) / scale
        assert err <= 1e-10, f"{what}: field {name} differs by {err:.3e} of its scale"


@pytest.mark.parametrize("rows,cols,nodes", [(1, 1, 40), (2, 3, 200)])
def test_mas_update_and_push_match_oracle(oracle_lib, rows, cols, nodes):
    w, grid, f0, f1 = _case(rows, cols, nodes)
    s0, k0 = W.mas_slice_struct(grid, f0)
    s1, k1 = W.mas_slice_struct(grid, f1)
    s_cor, phi_off = 0.37, 0.21
    mas = O.MasState(O.C.pointer(s0), O.C.pointer(s1), s_cor, phi_off, grid.params)
    d = w.dims()
    nodes_ref = W.initial_nodes(w)
    r_au = nodes_ref[abi.NODE["RMAG"]] * w.params.r_scale
    run = EpremRun(d, w.params, W.build_grids(w))
    run.upload_nodes(nodes_ref)
    run.mas_init(grid.params)
    run.mas_load_slice(2, s0)
    run.mas_load_slice(0, s1)
    run.mas_select(2, 0, s_cor, phi_off)

    oracle_lib.mas_update_mhd(d, w.params, nodes_ref, mas)
    run.update_mhd(0.0)
    inside = r_au <= grid.params.radial_max * W.RSAU
    assert inside.any() and (~inside).any()
    _assert_nodes_close(run.download_nodes(), nodes_ref, "masGetNode")
    for step in range(3):
        oracle_lib.mas_move_nodes(d, w.params, nodes_ref, mas, w.params.t_del)
        oracle_lib.mas_update_mhd(d, w.params, nodes_ref, mas, w.params.t_del)
        run.mas_move_nodes(w.params.t_del)
        run.update_mhd(w.params.t_del)
        _assert_nodes_close(run.download_nodes(), nodes_ref, f"RK4 step {step}")
    run.close()


def test_mas_requires_selection():
    w, grid, f0, f1 = _case()
    run = EpremRun(w.dims(), w.params, W.build_grids(w))
    run.upload_nodes(W.initial_nodes(w))
    run.mas_init(grid.params)
    with pytest.raises(Exception):
        run.mas_move_nodes(w.params.t_del)
    s0, k0 = W.mas_slice_struct(grid, f0)
    run.mas_load_slice(0, s0)
    with pytest.raises(Exception):
        run.mas_select(0, 1, 0.5)  # slot 1 never loaded
    with pytest.raises(Exception):
        run.mas_load_slice(5, s0)  # beyond max_slices
    run.close()


def test_mas_use_switches_back_to_the_analytic_wind(oracle_lib):
    """mhdGridStatus == MHD_DEFAULT before the first MAS time: updateMhd takes
    the analytic background although the slots stay loaded."""
    w, grid, f0, f1 = _case()
    s0, k0 = W.mas_slice_struct(grid, f0)
    d = w.dims()
    nodes = W.initial_nodes(w)
    run = EpremRun(d, w.params, W.build_grids(w))
    run.upload_nodes(nodes)
    run.mas_init(grid.params)
    run.mas_load_slice(0, s0)
    run.mas_select(0, 0, 0.0)
    run.mas_use(False)
    run.update_mhd(0.0)
    oracle_lib.update_mhd(d, w.params, nodes, 0.0)
    _assert_nodes_close(run.download_nodes(), nodes, "analytic after mas_use(False)")
    run.close()


def test_async_slice_loads_equal_synchronous_loads():
    """Slices queued on the copy stream (eprem_gpu_mas_load_slice_async) give
    the same background as synchronous loads, bit for bit, including a load
    into the third slot while the first pair is selected and in use, and a
    reload of a slot (its arrays kept, no reallocation); loading into a
    selected slot is refused."""
    w, grid, f0, f1 = _case(2, 2, 120)
    f2 = grid.slice_fields(grid.times[2])
    structs = [W.mas_slice_struct(grid, f) for f in (f0, f1, f2)]
    runs = []
    for mode in ("sync", "async"):
        run = EpremRun(w.dims(), w.params, W.build_grids(w))
        run.upload_nodes(W.initial_nodes(w))
        run.mas_init(grid.params)
        load = run.mas_load_slice if mode == "sync" else run.mas_load_slice_async
        load(0, structs[0][0])
        load(1, structs[1][0])
        run.mas_select(0, 1, 0.4, 0.1)
        if mode == "async":
            with pytest.raises(Exception):
                run.mas_load_slice_async(0, structs[0][0])
        run.update_mhd(0.0)
        run.mas_move_nodes(w.params.t_del)
        load(2, structs[2][0])  # the next slice while the pair is in use
        run.mas_select(1, 2, 0.2, 0.1)
        run.update_mhd(w.params.t_del)
        run.mas_move_nodes(w.params.t_del)
        load(0, structs[0][0])  # a reload of a slot that was read before
        run.mas_select(2, 0, 0.7, 0.1)
        run.update_mhd(2 * w.params.t_del)
        runs.append(run.download_nodes())
        run.close()
    a, b = runs
    same = (a == b) | (np.isnan(a) & np.isnan(b))
    assert same.all()
