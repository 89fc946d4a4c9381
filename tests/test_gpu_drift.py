"""Drift on the GPU (eprem_gpu_set_drift) against the oracle, through the C
ABI.  The oracle's curlBoverB2 / DriftShellData restatement is pinned bit for
bit to the reference (test_oracle_vs_reference.py, drift cases; whole runs in
test_drift_whole_run.py).  The GPU forms curl(B)/B^2 in its updateMhd and
gathers each cell's drift hand-overs in the reference's order without fused
multiply-adds; curl goes through CUDA's acos / sin, so the FP64 form is held
to the plain form's 1e-12 relative bound on f rather than bit equality.  The
FP32 form: omnidirectional flux within 1e-3 at J > 1e-30 max J."""
import numpy as np
import pytest

from eprem_gb300 import EpremRun, abi, workloads as W

from helpers import rel_err

pytestmark = pytest.mark.gpu


def random_news(S, seed):
    rng = np.random.default_rng(seed)
    news = rng.integers(0, S - 1, size=(S, 4))
    news += news >= np.arange(S)[:, None]
    return news.astype(np.int32)


def primed(orc, w, with_curl=True):
    """Nodes primed as the driver does (updateMhd, moveNodes, updateMhd) on
    the oracle, with curl(B)/B^2, and the seed distribution."""
    d = w.dims()
    g = W.build_grids(w)
    nodes = W.initial_nodes(w)
    curl = np.zeros((3, d.num_streams * d.num_nodes)) if with_curl else None
    orc.update_mhd(d, w.params, nodes, 0.0, curl)
    orc.move_nodes(d, w.params, nodes, w.params.t_del)
    orc.update_mhd(d, w.params, nodes, w.params.t_del, curl)
    return d, g, nodes, curl, W.initial_f(w, nodes, g)


def gpu_drift_run(w, precision, g, news, kp, calls):
    """The GPU run primed on the GPU (its own curl), then `calls` updates."""
    run = EpremRun(w.dims(precision), w.params, g)
    run.set_drift(news, W.drift_params(w, g))
    if kp is not None:
        run.set_shell_diffusion(news, kp)
    run.upload_nodes(W.initial_nodes(w))
    run.update_mhd(0.0)
    run.move_nodes(w.params.t_del)
    run.update_mhd(w.params.t_del)
    return run


CASES = {
    "2x2 faces, random links": (lambda: W.custom(2, 2, 40, 10, 8, num_ep_steps=3), None, 2),
    "3x3 faces, with shell diffusion": (lambda: W.custom(3, 3, 60, 9, 7, num_ep_steps=2), 0.05, 1),
    "cone-like, ideal shock": (lambda: W.testsuite_like("cone", 2, 2, 60), None, 2),
}


@pytest.mark.parametrize("name", list(CASES))
def test_fp64_drift_matches_oracle(name, oracle_lib):
    make, kp, calls = CASES[name]
    w = make()
    d, g, nodes, curl, f = primed(oracle_lib, w)
    news = random_news(d.num_streams, seed=len(name))
    dp = W.drift_params(w, g)
    gs, keep = W.grids_struct(g)
    f_ref, n_ref = f.copy(), nodes.copy()
    for _ in range(calls):
        rc, st, err = oracle_lib.update_energetic_particles_perp(d, w.params, gs, f_ref, n_ref,
                                                                 news, kp, dp, curl, nthreads=8)
        assert rc == 0, err
    run = gpu_drift_run(w, abi.EPREM_FP64, g, news, kp, calls)
    got = run.download_nodes()
    for fld in ("RX", "RY", "RZ", "RMAG", "BMAG"):
        np.testing.assert_allclose(got[abi.NODE[fld]], nodes[abi.NODE[fld]], rtol=1e-13,
                                   err_msg=fld)
    run.upload_f(f)
    for _ in range(calls):
        run.update_energetic_particles(0.0)
    st = run.read_stats()
    out = run.download_f()
    run.close()
    assert rel_err(out, f_ref) <= 1e-12
    # the drift is not a no-op here
    f_plain, n_plain = f.copy(), nodes.copy()
    for _ in range(calls):
        if kp is None:
            oracle_lib.update_energetic_particles(d, w.params, gs, f_plain, n_plain)
        else:
            oracle_lib.update_energetic_particles(d, w.params, gs, f_plain, n_plain, news=news,
                                                  kperxkpar=kp)
    assert rel_err(out, f_plain) > 1e-6


def test_fp32_drift_flux_within_1e3(oracle_lib):
    w = W.custom(2, 2, 100, 20, 20, num_ep_steps=3)
    d, g, nodes, curl, f = primed(oracle_lib, w)
    news = random_news(d.num_streams, seed=5)
    gs, keep = W.grids_struct(g)
    f_ref, n_ref = f.copy(), nodes.copy()
    for _ in range(2):
        rc, _, err = oracle_lib.update_energetic_particles_perp(
            d, w.params, gs, f_ref, n_ref, news, None, W.drift_params(w, g), curl, nthreads=8)
        assert rc == 0, err
    j_ref = oracle_lib.omni_flux(d, gs, f_ref)
    run = gpu_drift_run(w, abi.EPREM_FP32, g, news, None, 2)
    run.upload_f(f)
    for _ in range(2):
        run.update_energetic_particles(0.0)
    run.read_stats()
    j = run.omni_flux()
    run.close()
    mask = j_ref > 1e-30 * j_ref.max()
    assert float(np.max(np.abs(j[mask] - j_ref[mask]) / j_ref[mask])) <= 1e-3


def test_drift_switches_off_and_refuses_mas(oracle_lib):
    w = W.custom(1, 1, 30, 6, 6, num_ep_steps=2)
    d, g, nodes, _, f = primed(oracle_lib, w, with_curl=False)
    news = random_news(d.num_streams, seed=2)
    run = EpremRun(d, w.params, g)
    run.set_drift(news, W.drift_params(w, g))
    run.set_drift(None, None)  # off again: the plain update
    run.upload_nodes(nodes)
    run.upload_f(f)
    run.update_energetic_particles(0.0)
    out = run.download_f()
    f_ref, n_ref = f.copy(), nodes.copy()
    gs, keep = W.grids_struct(g)
    oracle_lib.update_energetic_particles(d, w.params, gs, f_ref, n_ref)
    assert rel_err(out, f_ref) <= 1e-12
    grid = W.mas_grid(nr=16, nt=8, np_=16, n_slices=2)
    run.mas_init(grid.params)
    with pytest.raises(Exception):
        run.set_drift(news, W.drift_params(w, g))
    run.close()
