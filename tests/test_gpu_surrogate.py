"""The split form and the learned surrogate, through the C ABI.

* the GPU forward / backward kernels (tcgen05 GEMMs + elementwise kernels)
  against the CPU statement of the network (oracle/mlp_oracle.py) with the
  same bf16 operand roundings;
* the split form (relaxation moved from the streaming sub-cycles to one
  exact step after the focusing) conserves sum_mu f; its flux error against
  the reference's unsplit FP64 form is measured;
* the surrogate of the focusing step conserves sum_mu f exactly;
* training on rows of a run's state reduces the loss; the trained surrogate
  keeps at least as many rows as an untrained one (which the residual check
  sends to the plain kernel), with the flux errors of both reported."""
import numpy as np
import pytest

import mlp_oracle as MO
from eprem_gb300 import EpremRun, abi, workloads as W
from eprem_gb300.runtime import (NODE_PHASE_SPLIT, NODE_PHASE_SURROGATE_FOCUS, Surrogate,
                                 set_node_phase, surrogate_counts)
from helpers import oracle_update, primed_state

pytestmark = pytest.mark.gpu


def _flux_err(a, b):
    mask = b > 1e-30 * b.max()
    return float(np.max(np.abs(a[mask] - b[mask]) / b[mask]))


def test_gradients_match_cpu_oracle():
    s = Surrogate(seed=3, chunk_rows=4096)
    p = s.get_params().astype(np.float64)
    rng = np.random.default_rng(11)
    x = rng.normal(0.0, 0.5, (256, 48)).astype(np.float32)
    x[:, 43:] = 0.0
    t = rng.normal(0.0, 0.05, (256, 40)).astype(np.float32)
    loss_g, g_g = s.loss_grad(x, t)
    loss_c, g_c = MO.loss_grad(p, x.astype(np.float64), t.astype(np.float64), rb=True)
    assert abs(loss_g - loss_c) <= 1e-3 * loss_c
    off = 0
    for name, shape in MO.SHAPES:
        n = int(np.prod(shape))
        a, b = g_g[off:off + n].astype(np.float64), g_c[off:off + n]
        rel = np.linalg.norm(a - b) / np.linalg.norm(b)
        assert rel <= 1e-2, f"{name}: relative gradient error {rel:.3e}"
        off += n
    y = s.evaluate(x).astype(np.float64)
    yc = MO.forward(MO.unpack(p), x.astype(np.float64))["y"]
    assert np.max(np.abs(y - yc)) <= 1e-2 * np.max(np.abs(yc))
    s.close()


def _run(w, orc, mode=None, surrogate=None):
    d, g, f, nodes = primed_state(w, orc, abi.EPREM_FP32)
    run = EpremRun(d, w.params, g)
    run.upload_f(f)
    run.upload_nodes(nodes)
    if mode is not None:
        set_node_phase(run, mode, surrogate)
    return run, (d, g, f, nodes)


def _mu_sums(f, w):
    return f.reshape(-1, w.num_mu).sum(axis=1)


def test_split_form_conserves_and_reports_its_error(oracle_lib):
    # node phase alone (no streaming, no change): focusing + relaxation
    # conserve sum_mu f in every row
    w0 = W.custom(1, 1, 120, 8, 40, num_ep_steps=2, use_parallel_diffusion=0,
                  use_adiabatic_change=0, check_seed_population=0)
    run, (d, g, f, nodes) = _run(w0, oracle_lib, NODE_PHASE_SPLIT)
    run.update_energetic_particles(0.0)
    got = run.download_f()
    s0, s1 = _mu_sums(f.astype(np.float32).astype(np.float64), w0), _mu_sums(got, w0)
    live = np.ones(s0.size, bool).reshape(w0.num_streams, w0.num_nodes, -1)
    live[:, 0, :] = False  # the spawn node is not updated
    assert np.max(np.abs(s1 - s0)[live.reshape(-1)] / s0[live.reshape(-1)]) <= 1e-5
    run.close()
    # full step: the split changes the reference's operator splitting; its
    # flux error against the unsplit FP64 form is measured, not bounded here
    w = W.custom(1, 1, 200, 10, 40, num_ep_steps=3)
    run, (d, g, f, nodes) = _run(w, oracle_lib, NODE_PHASE_SPLIT)
    f64, _, _ = oracle_update(oracle_lib, w, g, f, nodes)
    run.update_energetic_particles(0.0)
    gs, keep = W.grids_struct(g)
    err = _flux_err(run.omni_flux(), oracle_lib.omni_flux(w.dims(), gs, f64))
    print(f"split form flux error vs FP64 reference form: {err:.3e}")
    assert np.isfinite(err)
    run.close()


def test_surrogate_focus_conserves_particle_number(oracle_lib):
    """Focusing predicted by a (here untrained) network and projected: the
    row sums over mu stay those of the input, kept rows and fallen-back rows
    alike."""
    w = W.custom(1, 1, 120, 8, 40, num_ep_steps=2, use_parallel_diffusion=0,
                 use_adiabatic_change=0, check_seed_population=0)
    s = Surrogate(seed=9, chunk_rows=8192)
    s.set_tolerance(1e30)  # keep every finite row
    run, (d, g, f, nodes) = _run(w, oracle_lib, NODE_PHASE_SURROGATE_FOCUS, s)
    run.update_energetic_particles(0.0)
    kept, fb = surrogate_counts(run)
    assert kept > 0
    got = run.download_f()
    s0, s1 = _mu_sums(f.astype(np.float32).astype(np.float64), w), _mu_sums(got, w)
    live = np.ones((w.num_streams, w.num_nodes, w.num_energies), bool)
    live[:, 0, :] = False
    live = live.reshape(-1)
    assert np.max(np.abs(s1 - s0)[live] / s0[live]) <= 1e-5
    run.close()
    s.close()


def test_trained_surrogate_replaces_plain_rows(oracle_lib):
    w = W.custom(1, 2, 300, 12, 40, num_ep_steps=2)
    src, _ = _run(w, oracle_lib)
    s = Surrogate(seed=5, chunk_rows=16384)
    s.reserve(300000)
    n = 0
    for call in range(4):  # rows of a few successive states (focusing targets)
        n = s.collect(src, rate=1.0, seed=100 + call)
        src.update_energetic_particles(0.0)
    assert n > 100000
    l0 = s.train(1, 4096, 1e-3)
    l1 = s.train(3000, 4096, 1e-3)
    print(f"training loss {l0:.3e} -> {l1:.3e}")
    assert l1 < 0.5 * l0
    tol = s.calibrate(0.999, 1.5)
    assert tol > 0

    untrained = Surrogate(seed=6, chunk_rows=16384)
    untrained.set_tolerance(tol)
    plain, _ = _run(w, oracle_lib)  # the reference scheme, plain focusing
    sur, _ = _run(w, oracle_lib, NODE_PHASE_SURROGATE_FOCUS, s)
    raw, _ = _run(w, oracle_lib, NODE_PHASE_SURROGATE_FOCUS, untrained)
    for r in (plain, sur, raw):
        r.update_energetic_particles(0.0)
    rows = w.num_streams * (w.num_nodes - 1) * w.num_energies * w.params.num_ep_steps
    kept, fallback = surrogate_counts(sur)
    kept_raw, _ = surrogate_counts(raw)
    assert kept + fallback == rows
    j = plain.omni_flux()
    err = _flux_err(sur.omni_flux(), j)
    err_raw = _flux_err(raw.omni_flux(), j)
    print(f"trained: kept {kept}/{rows}, flux err {err:.3e}; untrained: kept {kept_raw}, "
          f"flux err {err_raw:.3e}")
    assert np.isfinite(err) and np.isfinite(err_raw)
    assert kept >= kept_raw
    for r in (src, plain, sur, raw):
        r.close()
    s.close()
    untrained.close()
