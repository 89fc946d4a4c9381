"""Ensembles, the autotuner and the device-side seed population, through the
C ABI.  An ensemble step is a graph replay of the same kernels the runs
launch one by one, so ensemble and individual stepping agree bit for bit."""
import numpy as np
import pytest

from eprem_gb300 import Ensemble, EpremRun, abi, workloads as W
from helpers import oracle_update, primed_state

pytestmark = pytest.mark.gpu


def _members():
    """Three runs of different sizes; the last has a moving ideal shock, so
    its updateMhd depends on the device-side time."""
    a = W.custom(1, 1, 120, 10, 8, num_ep_steps=3)
    b = W.custom(1, 2, 300, 6, 12, num_ep_steps=2)
    c = W.custom(2, 2, 80, 8, 10, num_ep_steps=2, ideal_shock=1, ideal_shock_speed=1500e5,
                 ideal_shock_init_time=0.0, ideal_shock_width=0.0)
    return [a, b, c]


def _start(w, orc, precision):
    d, g, f, nodes = primed_state(w, orc, precision)
    run = EpremRun(d, w.params, g)
    run.upload_f(f)
    run.upload_nodes(nodes)
    return run


@pytest.mark.parametrize("chains", [-1, 0, 1, 2])
@pytest.mark.parametrize("precision", [abi.EPREM_FP64, abi.EPREM_FP32])
def test_ensemble_step_equals_individual_steps(oracle_lib, precision, chains):
    """Every graph schedule (lock-step -- here, with unequal numEpSteps, one
    chain --, one branch per run, one serial chain, two chains) replays the
    runs' own kernels: bit-equal to stepping them."""
    ws = _members()
    td = ws[0].params.t_del
    t0 = [td, 2 * td, 3 * td]
    single = [_start(w, oracle_lib, precision) for w in ws]
    batched = [_start(w, oracle_lib, precision) for w in ws]
    for run, w, t in zip(single, ws, t0):
        for k in range(3):
            run.move_nodes(w.params.t_del)
            run.update_mhd(t + w.params.t_del)
            run.update_energetic_particles(t)
            t += w.params.t_del
        run.synchronize()
    ens = Ensemble(batched)
    ens.set_chains(chains)
    ens.set_time(t0)
    n0 = [r.kernel_launches for r in batched]
    for _ in range(3):
        ens.step()
    ens.synchronize()
    np.testing.assert_allclose(ens.get_time(), [t + 3 * w.params.t_del for t, w in zip(t0, ws)],
                               rtol=1e-15)
    for rs, rb, nb in zip(single, batched, n0):
        np.testing.assert_array_equal(rb.download_f(), rs.download_f())
        np.testing.assert_array_equal(rb.download_nodes(), rs.download_nodes())
        assert rb.read_stats().as_dict() == rs.read_stats().as_dict()
        assert rb.kernel_launches - nb > 0
    ens.close()
    for r in single + batched:
        r.close()


def _lockstep_members():
    """Runs with the same numEpSteps: two sharing the mu = 8 packed kernel,
    two sharing the mu = 40 one (one with a cluster of CTAs per slab), one
    with an ideal shock."""
    return [W.custom(1, 1, 120, 10, 8, num_ep_steps=2),
            W.custom(1, 2, 300, 6, 8, num_ep_steps=2),
            W.custom(2, 2, 80, 8, 40, num_ep_steps=2, ideal_shock=1, ideal_shock_speed=1500e5,
                     ideal_shock_init_time=0.0, ideal_shock_width=0.0),
            W.custom(1, 1, 1100, 5, 40, num_ep_steps=2)]


@pytest.mark.parametrize("precision", [abi.EPREM_FP64, abi.EPREM_FP32])
def test_lockstep_ensemble_equals_individual_steps(oracle_lib, precision):
    """The lock-step schedule (the default): sub-step by sub-step, the
    streaming of runs that share a packed kernel in one launch over all
    their slabs, longest first -- bit-equal to stepping each run alone."""
    ws = _lockstep_members()
    td = ws[0].params.t_del
    single = [_start(w, oracle_lib, precision) for w in ws]
    batched = [_start(w, oracle_lib, precision) for w in ws]
    for run, w in zip(single, ws):
        t = td
        for k in range(3):
            run.move_nodes(w.params.t_del)
            run.update_mhd(t + w.params.t_del)
            run.update_energetic_particles(t)
            t += w.params.t_del
        run.synchronize()
    ens = Ensemble(batched)
    ens.set_time([td] * len(ws))
    for _ in range(3):
        ens.step()
    ens.synchronize()
    for rs, rb in zip(single, batched):
        np.testing.assert_array_equal(rb.download_f(), rs.download_f())
        np.testing.assert_array_equal(rb.download_nodes(), rs.download_nodes())
        assert rb.read_stats().as_dict() == rs.read_stats().as_dict()
    ens.close()
    for r in single + batched:
        r.close()


def test_ensemble_refuses_mas_runs_and_duplicates(oracle_lib):
    w = W.custom(1, 1, 40, 4, 6)
    run = _start(w, oracle_lib, abi.EPREM_FP64)
    with pytest.raises(Exception):
        Ensemble([run, run])
    grid = W.mas_grid(nr=12, nt=8, np_=16, n_slices=2, r_max_rs=20.0)
    run.mas_init(grid.params)
    with pytest.raises(Exception):
        Ensemble([run])
    run.close()


def test_seed_population_on_device_matches_host_generator(oracle_lib):
    w = W.custom(1, 2, 90, 7, 6)
    d, g, f, nodes = primed_state(w, oracle_lib)
    run = EpremRun(d, w.params, g)
    run.upload_nodes(nodes)
    run.init_seed_population(w.seed, w.perturb)
    got = run.download_f()
    np.testing.assert_allclose(got, f, rtol=1e-13, atol=0.0)
    run.close()


def test_autotune_keeps_a_correct_shape(oracle_lib):
    w = W.custom(1, 1, 600, 6, 40, num_ep_steps=2, use_adiabatic_focus=0,
                 use_adiabatic_change=0)
    d, g, f, nodes = primed_state(w, oracle_lib, abi.EPREM_FP32)
    f_ref, _, _ = oracle_update(oracle_lib, w, g, f, nodes)
    run = EpremRun(d, w.params, g)
    run.upload_f(f)
    run.upload_nodes(nodes)
    v = run.autotune()
    assert v % 8 in (3, 4, 5, 6, 7) and 1 <= v // 8  # a kind and a CTA shape
    # the scratch copy leaves the state alone
    np.testing.assert_array_equal(run.download_f(), f.astype(np.float32).astype(np.float64))
    run.update_energetic_particles(0.0)
    got = run.download_f()
    assert np.max(np.abs(got - f_ref) / f_ref) <= 1e-3
    run.close()


def test_ensemble_autotune_by_size_class(oracle_lib):
    ws = _members()
    runs = [_start(w, oracle_lib, abi.EPREM_FP32) for w in ws]
    ens = Ensemble(runs)
    chosen = ens.autotune()
    assert len(chosen) == 3 and all(v % 8 in (3, 4, 5) and v // 8 >= 1 for v in chosen)
    ens.set_time(0.0)
    ens.step()
    ens.synchronize()
    for r in runs:
        assert np.all(np.isfinite(r.download_f()))
    ens.close()
    for r in runs:
        r.close()
