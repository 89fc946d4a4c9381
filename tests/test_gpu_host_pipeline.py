"""The host-buffer update (eprem_gpu_update_energetic_particles_host): the
streams go through in chunks whose copies overlap the neighbouring chunks'
updates.  Streams are independent on this path, so the result must be
bit-identical to uploading f, updating the whole run and downloading f."""
import numpy as np
import pytest

from eprem_gb300 import EpremGpuError, EpremRun, abi, workloads as W

from helpers import primed_state

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [abi.EPREM_FP64, abi.EPREM_FP32])
@pytest.mark.parametrize("in_place", [False, True])
def test_host_update_equals_whole_run_update(oracle_lib, precision, in_place):
    # 30 streams: chunks of 4, the last one of 2
    w = W.custom(1, 5, 60, 8, 8, num_ep_steps=2)
    d, g, f, nodes = primed_state(w, oracle_lib, precision)
    whole = EpremRun(d, w.params, g)
    whole.upload_f(f)
    whole.upload_nodes(nodes)
    whole.update_energetic_particles(0.0)
    st_w = whole.read_stats()
    f_w = whole.download_f()
    n_w = whole.download_nodes()
    whole.close()
    run = EpremRun(d, w.params, g)
    run.upload_nodes(nodes)
    f_in = f.copy()
    f_out = f_in if in_place else np.empty_like(f_in)
    run.update_energetic_particles_host(f_in, f_out, 0.0)
    st = run.read_stats()
    n_h = run.download_nodes()
    run.close()
    np.testing.assert_array_equal(f_out, f_w)
    np.testing.assert_array_equal(n_h, n_w)
    assert st.as_dict() == st_w.as_dict()
    if not in_place:
        np.testing.assert_array_equal(f_in, f)  # input untouched


def test_host_update_reports_the_run_stream(oracle_lib):
    """A NaN in a late chunk is reported at its stream number in the run."""
    w = W.custom(1, 5, 30, 8, 6, num_ep_steps=2)
    d, g, f, nodes = primed_state(w, oracle_lib)
    bad = f.copy()
    s_bad = 27  # chunk 6 of 8
    bad[((s_bad * 30 + 15) * 8 + 3) * 6 + 2] = np.nan
    run = EpremRun(d, w.params, g)
    run.upload_nodes(nodes)
    with pytest.raises(EpremGpuError) as ei:
        run.update_energetic_particles_host(bad, np.empty_like(bad), 0.0)
    assert ei.value.code == abi.EPREM_GPU_ERR_NAN
    assert f"stream {s_bad}" in str(ei.value), str(ei.value)
    run.close()


@pytest.mark.parametrize("precision", [abi.EPREM_FP64, abi.EPREM_FP32])
def test_host_update_with_a_stream_pitch(oracle_lib, precision):
    """f laid out as the reference's eParts: a ghost shell of E*M values
    before each stream's N shells (pitch (N+1)*E*M).  The result matches the
    contiguous call and the ghost shells stay as they were."""
    w = W.custom(1, 5, 60, 8, 8, num_ep_steps=2)
    d, g, f, nodes = primed_state(w, oracle_lib, precision)
    S, N, E, M = d.num_streams, d.num_nodes, d.num_energies, d.num_mu
    per, ghost = N * E * M, E * M
    pitch = per + ghost
    padded = np.full(S * pitch, -7.0)
    view = padded.reshape(S, pitch)
    view[:, ghost:] = f.reshape(S, per)
    run = EpremRun(d, w.params, g)
    run.upload_nodes(nodes)
    run.update_energetic_particles_host(padded[ghost:], padded[ghost:], 0.0, stream_pitch=pitch)
    st = run.read_stats()
    run.close()
    ref = EpremRun(d, w.params, g)
    ref.upload_nodes(nodes)
    f_ref = ref.update_energetic_particles_host(f.copy(), None, 0.0)
    st_ref = ref.read_stats()
    ref.close()
    np.testing.assert_array_equal(view[:, ghost:].reshape(-1), f_ref)
    assert np.all(view[:, :ghost] == -7.0)
    assert st.as_dict() == st_ref.as_dict()


def _as_stored(x, precision):
    """Values as the run holds them (FP32: float rounding; 2^64 shift exact)."""
    return x if precision == abi.EPREM_FP64 else x.astype(np.float32).astype(np.float64)


@pytest.mark.parametrize("precision", [abi.EPREM_FP64, abi.EPREM_FP32])
def test_pitched_f_round_trip_and_ripple(oracle_lib, precision):
    """eParts-shaped host f (a template row before each stream's N rows):
    pitched upload / download, and rippleShellsOut on the device -- node k
    takes node k-1, node 0 the stream's template row -- twice in a row."""
    w = W.custom(1, 2, 40, 6, 8, num_ep_steps=1)
    d, g, f, nodes = primed_state(w, oracle_lib, precision)
    S, N, E, M = d.num_streams, d.num_nodes, d.num_energies, d.num_mu
    em = E * M
    pitch = (N + 1) * em
    eparts = np.empty(S * pitch)
    view = eparts.reshape(S, N + 1, em)
    view[:, 1:, :] = f.reshape(S, N, em)
    rng = np.random.default_rng(3)
    view[:, 0, :] = rng.uniform(1e-6, 1e-3, (S, em))  # INNER_SHELL template rows
    run = EpremRun(d, w.params, g)
    run.upload_f_pitched(eparts[em:], pitch)
    back = np.full_like(eparts, -1.0)
    run.download_f_pitched(back[em:], pitch)
    np.testing.assert_array_equal(back.reshape(S, N + 1, em)[:, 1:, :],
                                  _as_stored(view[:, 1:, :], precision))
    assert np.all(back.reshape(S, N + 1, em)[:, 0, :] == -1.0)
    expect = view[:, 1:, :].copy()
    for _ in range(2):
        run.ripple_f(eparts, pitch)
        expect[:, 1:, :] = expect[:, :-1, :].copy()
        expect[:, 0, :] = view[:, 0, :]
    got = run.download_f().reshape(S, N, em)
    run.close()
    np.testing.assert_array_equal(got, _as_stored(expect, precision))
