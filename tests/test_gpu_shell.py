"""Cross-field (shell) diffusion on the GPU against the oracle, through the C
ABI (eprem_gpu_set_shell_diffusion).

The oracle's DiffuseShellData / ShellData restatement is pinned bit for bit to
the reference (test_oracle_vs_reference.py, the committed ref_shell_*.npz
outputs, and whole testsuite runs in test_shell_whole_run.py).  The GPU gathers
each cell's hand-overs in the reference's order without fused multiply-adds,
so the FP64 form must match within the plain form's 1e-12 relative bound on f;
the FP32 form within 1e-3 on the omnidirectional flux.  NEWS tables come from
the reference's own cube-sphere links (in the golden files) and from seeded
random tables, which also exercise repeated and one-way links.
"""
import glob
import os

import numpy as np
import pytest

from eprem_gb300 import EpremRun, Ensemble, EpremGpuError, abi, workloads as W

from helpers import primed_state, rel_err
from test_oracle_golden import load as load_golden

pytestmark = pytest.mark.gpu

F_RTOL = 1e-12
FLUX_RTOL = 1e-3
HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = sorted(glob.glob(os.path.join(HERE, "golden", "ref_shell_*.npz")))


def random_news(S, seed):
    """Seeded NEWS table without self-links (a self-link has zero length:
    the reference's ShellData divides by it)."""
    rng = np.random.default_rng(seed)
    news = rng.integers(0, S - 1, size=(S, 4))
    news += news >= np.arange(S)[:, None]  # skip the stream itself
    return news.astype(np.int32)


def oracle_shell(orc, w, g, f, nodes, news, kp, calls=1, dims=None):
    f = f.copy()
    nodes = nodes.copy()
    gs, keep = W.grids_struct(g)
    stats = []
    for _ in range(calls):
        rc, st, err = orc.update_energetic_particles(dims or w.dims(), w.params, gs, f, nodes,
                                                     nthreads=8, news=news, kperxkpar=kp)
        assert rc == 0, err
        stats.append(st)
    return f, nodes, stats


def gpu_shell(d, params, g, f, nodes, news, kp, calls=1):
    run = EpremRun(d, params, g)
    run.upload_f(f)
    run.upload_nodes(nodes)
    run.set_shell_diffusion(news, kp)
    stats = []
    for _ in range(calls):
        run.update_energetic_particles(0.0)
        stats.append(run.read_stats())
    out = run.download_f()
    run.close()
    return out, stats


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def test_fp64_matches_reference_outputs(path):
    """The reference's own outputs with its own NEWS links (one call)."""
    z, dims, params, g = load_golden(path)
    f_gpu, _ = gpu_shell(dims, params, g, z["f_in"], z["nodes_in"], z["news"],
                         float(z["kperxkpar"][0]))
    assert rel_err(f_gpu, z["f_out"]) <= F_RTOL


CASES = {
    "2x2 faces, random links": (lambda: W.custom(2, 2, 40, 10, 8, num_ep_steps=2), 1.0, 2),
    "4x4 faces, 200 nodes": (lambda: W.custom(4, 4, 200, 12, 10, num_ep_steps=2), 0.05, 1),
    "odd mu, capped": (lambda: W.custom(3, 3, 60, 9, 7, num_ep_steps=3), 50.0, 1),
    "wind-like 2x2": (lambda: W.testsuite_like("wind", 2, 2, 60), 0.05, 2),
}


@pytest.mark.parametrize("name", list(CASES))
def test_fp64_matches_oracle(name, oracle_lib):
    make, kp, calls = CASES[name]
    w = make()
    d, g, f, nodes = primed_state(w, oracle_lib)
    news = random_news(d.num_streams, seed=len(name))
    f_ref, _, st_ref = oracle_shell(oracle_lib, w, g, f, nodes, news, kp, calls)
    f_gpu, st_gpu = gpu_shell(d, w.params, g, f, nodes, news, kp, calls)
    assert rel_err(f_gpu, f_ref) <= F_RTOL
    for a, b in zip(st_gpu, st_ref):
        assert a.max_subcycles_focusing == b.max_subcycles_focusing
        assert a.max_subcycles_change == b.max_subcycles_change
    # the coupling is not a no-op here
    f_off, _ = gpu_shell(d, w.params, g, f, nodes, None, kp, calls)
    assert rel_err(f_off, f_ref) > 1e-6


def test_fp32_flux_within_1e3_of_oracle(oracle_lib):
    w = W.custom(2, 2, 100, 20, 20, num_ep_steps=3)
    d, g, f, nodes = primed_state(w, oracle_lib)
    news = random_news(d.num_streams, seed=7)
    f_ref, _, _ = oracle_shell(oracle_lib, w, g, f, nodes, news, 0.2, calls=2)
    gs, keep = W.grids_struct(g)
    j_ref = oracle_lib.omni_flux(d, gs, f_ref)
    run = EpremRun(w.dims(abi.EPREM_FP32), w.params, g)
    run.upload_f(f)
    run.upload_nodes(nodes)
    run.set_shell_diffusion(news, 0.2)
    for _ in range(2):
        run.update_energetic_particles(0.0)
    run.read_stats()
    j = run.omni_flux()
    run.close()
    mask = j_ref > 1e-30 * j_ref.max()
    assert float(np.max(np.abs(j[mask] - j_ref[mask]) / j_ref[mask])) <= FLUX_RTOL


@pytest.mark.parametrize("precision", [abi.EPREM_FP64, abi.EPREM_FP32])
def test_shell_diffusion_alone_conserves_particles(oracle_lib, precision):
    """With streaming, focusing, change and the seed check off, each sub-step
    only hands f between streams of a shell: every source's loss is the sum
    of the fractions its neighbours gain, so the sum over streams of every
    (node, energy, mu) cell is kept up to the rounding of the accumulation
    (FP32: the loss is the float sum of the float fractions)."""
    w = W.custom(2, 2, 40, 8, 6, num_ep_steps=4, use_parallel_diffusion=0,
                 use_adiabatic_focus=0, use_adiabatic_change=0, check_seed_population=0)
    d, g, f, nodes = primed_state(w, oracle_lib)
    news = random_news(d.num_streams, seed=11)
    out, _ = gpu_shell(w.dims(precision), w.params, g, f, nodes, news, 5.0, calls=2)
    shape = (d.num_streams, d.num_nodes, d.num_energies, d.num_mu)
    before = f.reshape(shape)[:, 1:].sum(axis=0)
    after = out.reshape(shape)[:, 1:].sum(axis=0)
    tol = 1e-13 if precision == abi.EPREM_FP64 else 1e-5
    assert np.max(np.abs(after - before) / before) <= tol
    assert rel_err(out, f) > 1e-4  # something moved


@pytest.mark.parametrize("precision", [abi.EPREM_FP64, abi.EPREM_FP32])
def test_host_update_equals_device_update(oracle_lib, precision):
    """With the streams coupled, the host-memory entry moves all of f at once;
    pitched host rows (the reference's eParts layout) included."""
    w = W.custom(2, 2, 50, 10, 8, num_ep_steps=2)
    d, g, f, nodes = primed_state(w, oracle_lib)
    dd = w.dims(precision)
    news = random_news(d.num_streams, seed=3)
    want, _ = gpu_shell(dd, w.params, g, f, nodes, news, 0.5)
    per = d.num_nodes * d.num_energies * d.num_mu
    pitch = per + d.num_energies * d.num_mu
    host = np.zeros(d.num_streams * pitch)
    host.reshape(d.num_streams, pitch)[:, :per] = f.reshape(d.num_streams, per)
    run = EpremRun(dd, w.params, g)
    run.upload_nodes(nodes)
    run.set_shell_diffusion(news, 0.5)
    run.update_energetic_particles_host(host, host, t_global=0.0, stream_pitch=pitch)
    run.close()
    got = host.reshape(d.num_streams, pitch)[:, :per].ravel()
    np.testing.assert_array_equal(got, want)


def test_switching_off_restores_the_plain_update(oracle_lib):
    w = W.custom(2, 2, 30, 8, 6, num_ep_steps=2)
    d, g, f, nodes = primed_state(w, oracle_lib)
    plain, _ = gpu_shell(d, w.params, g, f, nodes, None, 0.0)
    run = EpremRun(d, w.params, g)
    run.upload_f(f)
    run.upload_nodes(nodes)
    run.set_shell_diffusion(random_news(d.num_streams, 1), 0.5)
    run.set_shell_diffusion(None)
    run.update_energetic_particles(0.0)
    got = run.download_f()
    run.close()
    np.testing.assert_array_equal(got, plain)


def test_zero_length_link_is_reported_as_nan(oracle_lib):
    """A stream linked to itself has dl = 0; ShellData's division makes dlPer
    NaN and DiffuseShellData's checkNaN panics -- the same failure here."""
    w = W.custom(2, 2, 30, 8, 6, num_ep_steps=2)
    d, g, f, nodes = primed_state(w, oracle_lib)
    news = random_news(d.num_streams, 5)
    news[3, 1] = 3
    run = EpremRun(d, w.params, g)
    run.upload_f(f)
    run.upload_nodes(nodes)
    run.set_shell_diffusion(news, 0.5)
    run.update_energetic_particles(0.0)
    with pytest.raises(EpremGpuError) as ei:
        run.read_stats()
    run.close()
    assert ei.value.code == abi.EPREM_GPU_ERR_NAN
    assert "DiffuseShellData" in str(ei.value)
    gs, keep = W.grids_struct(g)
    rc, _, err = oracle_lib.update_energetic_particles(d, w.params, gs, f.copy(), nodes.copy(),
                                                       news=news, kperxkpar=0.5)
    assert rc == abi.EPREM_GPU_ERR_NAN and "DiffuseShellData" in err


def test_bad_arguments_and_ensembles_are_refused(oracle_lib):
    w = W.custom(2, 2, 30, 8, 6, num_ep_steps=2)
    d, g, f, nodes = primed_state(w, oracle_lib)
    run = EpremRun(d, w.params, g)
    bad = random_news(d.num_streams, 2)
    bad[0, 0] = d.num_streams
    with pytest.raises(EpremGpuError) as ei:
        run.set_shell_diffusion(bad, 0.5)
    assert ei.value.code == abi.EPREM_GPU_ERR_ARG
    with pytest.raises(EpremGpuError) as ei:
        run.set_shell_diffusion(random_news(d.num_streams, 2), 0.0)
    assert ei.value.code == abi.EPREM_GPU_ERR_ARG
    run.set_shell_diffusion(random_news(d.num_streams, 2), 0.5)
    with pytest.raises(EpremGpuError) as ei:
        Ensemble([run])
    assert ei.value.code == abi.EPREM_GPU_ERR_UNSUPPORTED
    run.close()
