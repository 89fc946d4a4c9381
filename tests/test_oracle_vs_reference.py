"""The oracle against the reference's own C, live: both run on the same state
and must agree bit for bit.  Needs oracle/_ref/libeprem_ref.so (built from the
reference source tree by oracle/Makefile where that tree exists); skipped
elsewhere -- the committed golden vectors cover that case."""
import multiprocessing as mp
import os

import numpy as np
import pytest

import oracle as O
from eprem_gb300 import abi, workloads as W

pytestmark = pytest.mark.skipif(not os.path.exists(O.REF_LIB),
                                reason="reference harness not built here")

def _scale_per_stream():
    """The precision-at-scale workload's streams (1000 nodes, 50 energies to
    1000 MeV, 40 mu) on 6 of them, for 3 EP sub-steps of the full call's
    sub-step length (up to 567 streaming sub-cycles each)."""
    w = W.with_faces(W.scale_plain(), 1, 1)
    w.params.t_del = w.params.t_del / w.params.num_ep_steps * 3
    w.params.num_ep_steps = 3
    return w


CASES = {
    "wind_like_thinned": lambda: W.testsuite_like("wind", 1, 1, 30),
    "cone_like_shock": lambda: W.testsuite_like("cone", 1, 1, 40),
    "plain_2x2_faces": lambda: W.custom(2, 2, 24, 10, 8, num_ep_steps=3),
    "alg2": lambda: W.custom(1, 1, 30, 10, 8, num_ep_steps=3, adiabatic_focus_alg=2,
                             adiabatic_change_alg=2),
    "alg3": lambda: W.custom(1, 1, 30, 10, 8, num_ep_steps=3, adiabatic_focus_alg=3,
                             adiabatic_change_alg=3),
    "mfpB_damped_noseedcheck": lambda: W.custom(1, 1, 30, 10, 8, num_ep_steps=3, mfp_type=2,
                                                damp_cooling=0.4, check_seed_population=0),
    "no_boundary_odd_mu": lambda: W.custom(1, 1, 30, 9, 7, num_ep_steps=3, use_ep_boundary=0),
    # the CPU-runnable plain workload at its full size (24 x 400 x 20 x 20, 30
    # EP sub-steps per call), whose whole 24 h run the GPU is checked against
    "cpu_runnable_full_size": W.small_plain,
    "precision_at_scale_streams": _scale_per_stream,
    # shell diffusion (DiffuseShellData) on the reference's own NEWS links
    "shell_1x1_faces": lambda: W.custom(1, 1, 20, 8, 6, num_ep_steps=2),
    "shell_2x2_faces": lambda: W.custom(2, 2, 24, 10, 8, num_ep_steps=3),
    "shell_3x2_capped_alg3": lambda: W.custom(3, 2, 16, 6, 6, num_ep_steps=2,
                                              adiabatic_focus_alg=3, adiabatic_change_alg=3),
}
SHELL = {"shell_1x1_faces": 0.5, "shell_2x2_faces": 0.05, "shell_3x2_capped_alg3": 50.0,
         "drift_shell_3x2": 0.05}
# drift (DriftShellData with curlBoverB2 from the analytic updateMhd), alone,
# with shell diffusion, and through the ideal shock
CASES.update({
    "drift_2x2_faces": lambda: W.custom(2, 2, 24, 10, 8, num_ep_steps=3),
    "drift_shell_3x2": lambda: W.custom(3, 2, 16, 8, 6, num_ep_steps=2),
    "drift_cone_shock": lambda: W.testsuite_like("cone", 1, 1, 40),
})
DRIFT = {"drift_2x2_faces", "drift_shell_3x2", "drift_cone_shock"}


def _reference_run(name, q):
    w = CASES[name]()
    ref = O.Reference()
    g = ref.setup(w)
    news = ref.shell_diffusion(SHELL[name], w.dims().num_streams) if name in SHELL else None
    lnpmin = None
    if name in DRIFT:
        news, lnpmin = ref.drift(w.dims().num_streams)
    nodes0 = W.initial_nodes(w)
    f0 = np.zeros(w.cells)
    ref.load(f0, nodes0)
    ref.update_mhd(0.0)
    ref.move_nodes(w.params.t_del)
    ref.update_mhd(w.params.t_del)
    nodes_in = np.zeros_like(nodes0)
    ref.store(f0, nodes_in)
    f_in = W.initial_f(w, nodes_in, g)
    ref.load(f_in, nodes_in)
    outs = []
    for _ in range(2):  # two calls: state carried over as the driver does
        rc, st = ref.update_energetic_particles(0.0)
        outs.append((rc, st.max_subcycles_change, st.max_subcycles_focusing, st.min_tau))
    f_out = np.zeros_like(f_in)
    nodes_out = np.zeros_like(nodes_in)
    ref.store(f_out, nodes_out)
    q.put((g, nodes0, nodes_in, f_in, f_out, nodes_out, outs, news, lnpmin))


@pytest.mark.parametrize("name", list(CASES))
def test_oracle_bit_exact_with_reference(name, oracle_lib):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    p = ctx.Process(target=_reference_run, args=(name, q))
    p.start()
    g_ref, nodes0, nodes_in_ref, f_in, f_out_ref, nodes_out_ref, outs, news, lnpmin = q.get(
        timeout=300)
    p.join()
    w = CASES[name]()
    g = oracle_lib.grids(w.num_energies, w.num_mu, w.e_min, w.e_max, w.mass, w.charge,
                         w.rigidity_power)
    for k in ("egrid", "vgrid", "vgrid_i", "mugrid", "rigidity", "dlnp", "dmu"):
        assert np.array_equal(np.asarray(g[k]), np.asarray(g_ref[k])), k
    d = w.dims()
    nodes = nodes0.copy()
    curl = np.zeros((3, d.num_streams * d.num_nodes)) if name in DRIFT else None
    oracle_lib.update_mhd(d, w.params, nodes, 0.0, curl)
    oracle_lib.move_nodes(d, w.params, nodes, w.params.t_del)
    oracle_lib.update_mhd(d, w.params, nodes, w.params.t_del, curl)
    assert np.array_equal(nodes, nodes_in_ref)
    gs, keep = W.grids_struct(g)
    f = f_in.copy()
    if name in DRIFT:
        assert lnpmin == W.build_grids(w)["lnpmin"]
        dp = W.drift_params(w, W.build_grids(w))
        assert np.any(curl != 0.0)
    for call in range(2):
        if name in DRIFT:
            rc, st, err = oracle_lib.update_energetic_particles_perp(
                d, w.params, gs, f, nodes, news, SHELL.get(name), dp, curl)
        else:
            shell = {} if news is None else {"news": news, "kperxkpar": SHELL[name]}
            rc, st, err = oracle_lib.update_energetic_particles(d, w.params, gs, f, nodes,
                                                                **shell)
        assert rc == outs[call][0] == 0, err
        assert (st.max_subcycles_change, st.max_subcycles_focusing) == outs[call][1:3]
        assert st.min_tau == outs[call][3]
    assert np.array_equal(f, f_out_ref)
    assert np.array_equal(nodes, nodes_out_ref)
