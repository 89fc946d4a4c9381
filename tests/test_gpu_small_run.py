"""The CPU-runnable plain-method workload at full size on the GPU: 24 streams
x 400 nodes x 20 energies x 20 mu through the driver's whole 24 h (96 steps
of moveNodes + updateMhd + updateEnergeticParticles, 30 EP sub-steps each,
2880 sub-steps), FP64 form, through the C ABI, against the oracle's run of the
same state recorded in tests/golden/small_run_24h.npz
(tests/golden/make_small_run.py):
  * every step's sub-cycle maxima and cell x sub-cycle counts equal, min tau
    within 1e-13;
  * f of stream 0 within 1e-12 relative, and the per-(stream, node) and
    per-(stream, energy, mu) sums of f of every stream within 1e-12.
"""
import os

import numpy as np
import pytest

from eprem_gb300 import EpremRun, abi, workloads as W

from helpers import primed_state

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "small_run_24h.npz")


def test_small_workload_whole_run_matches_oracle(oracle_lib):
    z = np.load(GOLDEN)
    fields = [str(s) for s in z["stat_fields"]]
    w = W.small_plain()
    d, g, f, nodes = primed_state(w, oracle_lib)
    run = EpremRun(d, w.params, g)
    run.upload_f(f)
    run.upload_nodes(nodes)
    dt = w.params.t_del
    t = dt
    stats = []
    for _ in range(len(z["stats"])):
        run.move_nodes(dt)
        run.update_mhd(t + dt)
        run.update_energetic_particles(t)
        st = run.read_stats()
        stats.append([getattr(st, n) for n in fields])
        t += dt
    out = run.download_f()
    run.close()
    stats = np.array(stats)
    want = z["stats"]
    for i, name in enumerate(fields):
        if name == "min_tau":
            np.testing.assert_allclose(stats[:, i], want[:, i], rtol=1e-13, err_msg=name)
        else:
            np.testing.assert_array_equal(stats[:, i], want[:, i], err_msg=name)
    S, N, E, M = d.num_streams, d.num_nodes, d.num_energies, d.num_mu
    f4 = out.reshape(S, N, E, M)
    ref0 = z["f_stream0"]
    assert np.max(np.abs(f4[0] - ref0) / ref0) <= 1e-12
    for key, got in (("sum_sn", f4.sum(axis=(2, 3))), ("sum_sem", f4.sum(axis=1))):
        ref = z[key]
        assert np.max(np.abs(got - ref) / ref) <= 1e-12, key
