"""Failure detection without a GPU fault: bad inputs are made on the host and
the device reports them through its status word, as the reference's
checkNaN / checkInf / FindSegmentLengths panics would (src/error.c:57-102,
src/energeticParticles.c:2594-2595).  After a reported failure the run stays
usable."""
import numpy as np
import pytest

from eprem_gb300 import EpremGpuError, EpremRun, abi, workloads as W

from helpers import primed_state

pytestmark = pytest.mark.gpu


def _run(w, oracle_lib):
    d, g, f, nodes = primed_state(w, oracle_lib)
    run = EpremRun(d, w.params, g)
    run.upload_f(f)
    run.upload_nodes(nodes)
    return run, d, g, f, nodes


def test_nan_in_distribution_is_reported(oracle_lib):
    w = W.custom(1, 1, 30, 8, 6, num_ep_steps=2)
    run, d, g, f, nodes = _run(w, oracle_lib)
    bad = f.copy()
    # stream 1, node 15, energy 3, mu 2: an interior node (the first three
    # list nodes are reset to the seed every sub-cycle, which would erase it)
    bad[((1 * 30 + 15) * 8 + 3) * 6 + 2] = np.nan
    run.upload_f(bad)
    run.update_energetic_particles(0.0)
    with pytest.raises(EpremGpuError) as ei:
        run.read_stats()
    assert ei.value.code == abi.EPREM_GPU_ERR_NAN
    assert "NaN value in" in str(ei.value)
    # the oracle reports the same failure
    gs, keep = W.grids_struct(g)
    rc, _, err = oracle_lib.update_energetic_particles(d, w.params, gs, bad.copy(), nodes.copy())
    assert rc == abi.EPREM_GPU_ERR_NAN and "NaN" in err
    # the run recovers with good data
    run.upload_f(f)
    run.update_energetic_particles(0.0)
    run.read_stats()
    run.close()


def test_inf_in_distribution_is_reported(oracle_lib):
    w = W.custom(1, 1, 30, 8, 6, num_ep_steps=1, use_parallel_diffusion=0,
                 use_adiabatic_change=0)
    run, d, g, f, nodes = _run(w, oracle_lib)
    bad = f.copy()
    bad[(3 * 8 + 2) * 6 + 1] = np.inf  # node 3 (focused), energy 2
    run.upload_f(bad)
    run.update_energetic_particles(0.0)
    with pytest.raises(EpremGpuError) as ei:
        run.synchronize()
    assert ei.value.code in (abi.EPREM_GPU_ERR_INF, abi.EPREM_GPU_ERR_NAN)
    run.close()


def test_zero_segment_is_reported(oracle_lib):
    w = W.custom(1, 1, 30, 8, 6, num_ep_steps=1, dsh_min=-1.0)
    d, g, f, nodes = primed_state(w, oracle_lib)
    for fld in ("RX", "RY", "RZ", "RMAG"):  # node 11 on top of node 10
        nodes[abi.NODE[fld], 11] = nodes[abi.NODE[fld], 10]
    run = EpremRun(d, w.params, g)
    run.upload_f(f)
    run.upload_nodes(nodes)
    run.update_energetic_particles(0.0)
    with pytest.raises(EpremGpuError) as ei:
        run.read_stats()
    assert ei.value.code == abi.EPREM_GPU_ERR_DS
    assert "Underflow in ds" in str(ei.value)
    gs, keep = W.grids_struct(g)
    rc, _, err = oracle_lib.update_energetic_particles(d, w.params, gs, f.copy(), nodes.copy())
    assert rc == abi.EPREM_GPU_ERR_DS
    run.close()


def test_stream_thinned_below_three_nodes(oracle_lib):
    w = W.custom(1, 1, 30, 8, 6, num_ep_steps=1, dsh_min=1e9)
    run, d, g, f, nodes = _run(w, oracle_lib)
    run.update_energetic_particles(0.0)
    with pytest.raises(EpremGpuError) as ei:
        run.read_stats()
    assert ei.value.code == abi.EPREM_GPU_ERR_STATE
    run.close()


def test_subcycle_cap(oracle_lib):
    w = W.custom(1, 1, 30, 8, 6, num_ep_steps=1, max_subcycles=2)
    run, d, g, f, nodes = _run(w, oracle_lib)
    run.update_energetic_particles(0.0)
    with pytest.raises(EpremGpuError) as ei:
        run.read_stats()
    assert ei.value.code == abi.EPREM_GPU_ERR_SUBCYCLES
    run.close()


def test_unsupported_species_rejected_at_create():
    w = W.custom(1, 1, 30, 8, 6)
    d = w.dims()
    d.num_species = 2
    with pytest.raises(EpremGpuError) as ei:
        EpremRun(d, w.params, W.build_grids(w))
    assert ei.value.code == abi.EPREM_GPU_ERR_UNSUPPORTED


@pytest.mark.parametrize("precision", [abi.EPREM_FP64, abi.EPREM_FP32])
def test_nan_node_rate_leaves_the_node_as_the_reference_does(oracle_lib, precision):
    """A node whose DuPar is NaN has NaN face speeds everywhere: the
    reference's CFL maximum passes over them (fabs(NaN) > max is false), so
    its sub-cycle counts are zero and focusing and change leave the node as
    it is -- no panic.  The GPU forms do the same."""
    w = W.custom(1, 1, 30, 6, 6, num_ep_steps=2)
    d, g, f, nodes = primed_state(w, oracle_lib)
    nodes[abi.NODE["DUPAR"], 10] = np.nan
    f_ref, n_ref = f.copy(), nodes.copy()
    gs, keep = W.grids_struct(g)
    rc, st, err = oracle_lib.update_energetic_particles(d, w.params, gs, f_ref, n_ref)
    assert rc == 0, err
    run = EpremRun(w.dims(precision), w.params, g)
    run.upload_f(f)
    run.upload_nodes(nodes)
    run.update_energetic_particles(0.0)
    run.read_stats()
    out = run.download_f()
    run.close()
    assert np.all(np.isfinite(out))
    tol = 1e-12 if precision == abi.EPREM_FP64 else 1e-3
    assert np.max(np.abs(out - f_ref) / f_ref) <= tol
