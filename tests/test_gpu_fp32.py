"""The FP32 form: f and the stencil / scattering arithmetic in float, node
geometry, dt and CFL in double.  Its omnidirectional flux must stay within
1e-3 relative of the FP64 result (the metric's accuracy bar), counted over
(node, energy) with J above 1e-30 of the maximum."""
import numpy as np
import pytest

from eprem_gb300 import EpremRun, abi, workloads as W

from helpers import oracle_update, primed_state

pytestmark = pytest.mark.gpu

FLUX_RTOL = 1e-3


def flux_err(j, jref):
    mask = jref > 1e-30 * jref.max()
    return float(np.max(np.abs(j[mask] - jref[mask]) / jref[mask]))


@pytest.mark.parametrize("calls", [1, 3])
def test_fp32_flux_within_1e3_of_oracle(oracle_lib, calls):
    w = W.custom(1, 1, 200, 20, 20)  # the small workload's slab shape, 30 sub-steps a call
    d, g, f, nodes = primed_state(w, oracle_lib)
    f_ref, _, _ = oracle_update(oracle_lib, w, g, f, nodes, calls=calls)
    gs, keep = W.grids_struct(g)
    j_ref = oracle_lib.omni_flux(d, gs, f_ref)
    run = EpremRun(w.dims(abi.EPREM_FP32), w.params, g)
    run.upload_f(f)
    run.upload_nodes(nodes)
    for _ in range(calls):
        run.update_energetic_particles(0.0)
    st = run.read_stats()
    j = run.omni_flux()
    run.close()
    assert flux_err(j, j_ref) <= FLUX_RTOL
    assert st.max_subcycles_focusing > 0


def test_fp32_sub_cycle_counts_equal_fp64(oracle_lib):
    """Sub-cycle counts come from FP64 geometry and CFL in both forms."""
    w = W.custom(1, 1, 60, 10, 8, num_ep_steps=2)
    d, g, f, nodes = primed_state(w, oracle_lib)
    _, _, stats = oracle_update(oracle_lib, w, g, f, nodes)
    run = EpremRun(w.dims(abi.EPREM_FP32), w.params, g)
    run.upload_f(f)
    run.upload_nodes(nodes)
    run.update_energetic_particles(0.0)
    st = run.read_stats()
    run.close()
    assert st.max_substeps_stream == stats[0].max_substeps_stream
    assert st.stream_cell_subcycles == stats[0].stream_cell_subcycles
    assert st.max_subcycles_focusing == stats[0].max_subcycles_focusing


@pytest.mark.parametrize("nodes", [400, 1100])
def test_fp32_streaming_shapes_agree(oracle_lib, nodes):
    """The FP32 streaming shapes (several nodes per thread; the same with
    packed fp32x2 arithmetic, with run-time or compile-time cell guards)
    compute the same update up to float rounding; 1100 nodes needs multi-CTA
    clusters (their common slab exponent is reduced across the cluster)."""
    w = W.custom(1, 1, nodes, 3, 40, num_ep_steps=2, use_adiabatic_focus=0,
                 use_adiabatic_change=0)
    d, g, f, nodes_arr = primed_state(w, oracle_lib)
    f_ref, _, _ = oracle_update(oracle_lib, w, g, f, nodes_arr)
    outs = []
    for variant in (3, 4, 5):
        w.params.stream_variant = variant
        run = EpremRun(w.dims(abi.EPREM_FP32), w.params, g)
        run.upload_f(f)
        run.upload_nodes(nodes_arr)
        run.update_energetic_particles(0.0)
        outs.append(run.download_f())
        run.close()
    w.params.stream_variant = 0
    # FP32 rounding accumulates over the streaming sub-cycles (several
    # hundred at 1100 nodes), most in the far tail of f
    for v, o in zip((3, 4, 5), outs):
        err = np.max(np.abs(o - f_ref) / f_ref)
        assert err <= 1e-3, f"variant {v} vs FP64 oracle: {err:.3e}"
    for v, o in zip((4, 5), outs[1:]):
        err = np.max(np.abs(o - outs[0]) / outs[0])
        assert err <= 1e-4, f"variant {v} vs variant 3: {err:.3e}"


@pytest.mark.parametrize("nodes,thin,seed_check,mu", [
    (48, 0, 1, 40), (401, 0, 1, 40), (402, 5, 0, 40), (403, 0, 0, 40), (1100, 0, 1, 40),
    (1500, 7, 1, 40), (400, 0, 1, 20), (447, 3, 0, 20), (1000, 0, 1, 20), (2000, 0, 1, 20)])
def test_fp32_mirrored_kinds_agree(oracle_lib, nodes, thin, seed_check, mu):
    """The mirrored streaming kinds (the mu < 0 half in mirror order, one
    upwind coefficient per two cells; 7 with the coefficients in shared memory
    and, on one CTA, the neighbour-warp halo hand-over) against the packed
    kind and the FP64 oracle.  The list lengths cover every position of the
    last list node modulo the nodes per thread (the slots start up to three
    nodes before list node 0), thinned streams, clusters of two and three
    CTAs, the seed check on and off, and both mu bins the mirrored kinds are
    built for (40; 20 with two-warp CTAs for short streams and float2 rows);
    both stream ends must keep the values the reference keeps."""
    w = W.custom(1, 1, nodes, 3, mu, num_ep_steps=2, use_adiabatic_focus=0,
                 use_adiabatic_change=0, check_seed_population=seed_check)
    w.cluster_inner = thin
    d, g, f, nodes_arr = primed_state(w, oracle_lib)
    f_ref, _, _ = oracle_update(oracle_lib, w, g, f, nodes_arr)
    outs = {}
    base = 5 if mu == 40 else 4  # the packed kind of the run's mu bin
    for variant in (base, 6, 7):
        w.params.stream_variant = variant
        run = EpremRun(w.dims(abi.EPREM_FP32), w.params, g)
        run.upload_f(f)
        run.upload_nodes(nodes_arr)
        run.update_energetic_particles(0.0)
        outs[variant] = run.download_f()
        run.close()
    w.params.stream_variant = 0
    for v, o in outs.items():
        err = np.max(np.abs(o - f_ref) / f_ref)
        assert err <= 1e-3, f"variant {v} vs FP64 oracle: {err:.3e}"
    for v in (6, 7):
        err = np.max(np.abs(outs[v] - outs[base]) / outs[base])
        assert err <= 1e-4, f"variant {v} vs variant {base}: {err:.3e}"


def test_fp32_mirrored_kinds_need_the_seed_boundary():
    """Without the seed boundary list node 0 has no fixed upwind value, so the
    mirrored kinds are refused and the automatic choice is the packed kind."""
    w = W.custom(1, 1, 100, 3, 40, use_ep_boundary=0)
    g = W.build_grids(w)
    for variant in (6, 7):
        w.params.stream_variant = variant
        with pytest.raises(RuntimeError):
            EpremRun(w.dims(abi.EPREM_FP32), w.params, g)
    w.params.stream_variant = 0
    EpremRun(w.dims(abi.EPREM_FP32), w.params, g).close()


def test_fp32_variants_of_the_fp64_kernel_refused():
    """Variants 1 and 2 name the FP64 streaming kernel's shape: an FP32 run
    refuses them instead of running another kernel."""
    w = W.custom(1, 1, 100, 3, 8)
    g = W.build_grids(w)
    for variant in (1, 2):
        w.params.stream_variant = variant
        with pytest.raises(RuntimeError):
            EpremRun(w.dims(abi.EPREM_FP32), w.params, g)
    w.params.stream_variant = 0


@pytest.mark.parametrize("cutoff_mev", [0.5, 0.25])
def test_fp32_row_exponents_hold_steep_spectra(oracle_lib, cutoff_mev):
    """A seed spectrum with an exponential cut-off (f falls as exp(-E/Ec):
    100 and 190 decades between the first and last energy rows)
    leaves the float range many times over.  With an exponent per (stream,
    node, energy) row the FP32 form keeps every row in range: flux within
    1e-3 of the FP64 oracle at J > 1e-30 max J, after three calls (90
    sub-steps), and f itself close to the oracle down to the reference's
    DBL_MIN floor wherever the oracle is above 1e-280."""
    w = W.custom(1, 1, 200, 20, 20)
    w.params.bf_ecutoff = cutoff_mev
    d, g, f, nodes = primed_state(w, oracle_lib)
    assert f.min() < 1e-80 * f.max()  # beyond any single float exponent range
    f_ref, _, _ = oracle_update(oracle_lib, w, g, f, nodes, calls=3)
    gs, keep = W.grids_struct(g)
    j_ref = oracle_lib.omni_flux(d, gs, f_ref)
    run = EpremRun(w.dims(abi.EPREM_FP32), w.params, g)
    run.upload_f(f)
    run.upload_nodes(nodes)
    for _ in range(3):
        run.update_energetic_particles(0.0)
    run.read_stats()
    j = run.omni_flux()
    f32 = run.download_f()
    run.close()
    assert flux_err(j, j_ref) <= FLUX_RTOL
    deep = f_ref > 1e-280
    assert np.max(np.abs(f32[deep] - f_ref[deep]) / f_ref[deep]) <= 1e-2


@pytest.mark.parametrize("mu", [6, 22, 23])
def test_fp32_packed_shape_with_odd_halves(oracle_lib, mu):
    """Odd numbers of cells per mu half (6: 3 + 3, 22: 11 + 11, 23: 11 + 12)
    take the packed shape with a zero padding cell: the same update as the
    scalar shape up to float rounding, and within 1e-3 of the FP64 oracle."""
    w = W.custom(1, 1, 300, 4, mu, num_ep_steps=2)
    d, g, f, nodes_arr = primed_state(w, oracle_lib)
    f_ref, _, _ = oracle_update(oracle_lib, w, g, f, nodes_arr)
    outs = {}
    for variant in (3, 4, 0):
        w.params.stream_variant = variant
        run = EpremRun(w.dims(abi.EPREM_FP32), w.params, g)
        run.upload_f(f)
        run.upload_nodes(nodes_arr)
        run.update_energetic_particles(0.0)
        run.read_stats()
        outs[variant] = run.download_f()
        run.close()
    w.params.stream_variant = 0
    np.testing.assert_array_equal(outs[0], outs[4])  # the automatic choice is the packed shape
    assert np.max(np.abs(outs[4] - outs[3]) / outs[3]) <= 1e-4
    assert np.max(np.abs(outs[4] - f_ref) / f_ref) <= 1e-3


def test_fp32_seed_check_without_streaming(oracle_lib):
    """seedPopulationCheck without parallel diffusion runs as its own kernel;
    in the FP32 form it renormalises each row it raises to the seed."""
    w = W.custom(1, 1, 80, 12, 10, num_ep_steps=3, use_parallel_diffusion=0)
    d, g, f, nodes = primed_state(w, oracle_lib)
    f = f * 1e-30  # far below the seed: every cell is raised
    f_ref, _, _ = oracle_update(oracle_lib, w, g, f, nodes)
    gs, keep = W.grids_struct(g)
    j_ref = oracle_lib.omni_flux(d, gs, f_ref)
    run = EpremRun(w.dims(abi.EPREM_FP32), w.params, g)
    run.upload_f(f)
    run.upload_nodes(nodes)
    run.update_energetic_particles(0.0)
    run.read_stats()
    j = run.omni_flux()
    run.close()
    assert flux_err(j, j_ref) <= FLUX_RTOL


def test_fp32_flux_within_1e3_over_driver_steps():
    """The per-stream workload of the 1536 x 1000 x 50 x 40 headline case (6
    streams) through six whole driver steps -- up to 567 streaming
    sub-cycles per EP sub-step, 30 sub-steps a step, 10^5 sub-cycles in all --
    in the FP32 and the FP64 form from the same state: the flux stays within
    1e-3.  Guards against any fixed per-sub-cycle bias: a relaxation whose
    two float factors missed a sum of 1 by 3e-8 drifted a node's particle
    number by 2e-3 over these steps."""
    w = W.with_faces(W.scale_plain(), 1, 1)
    g = W.build_grids(w)
    runs = []
    for precision in (abi.EPREM_FP64, abi.EPREM_FP32):
        run = EpremRun(w.dims(precision), w.params, g)
        run.upload_nodes(W.initial_nodes(w))
        run.update_mhd(0.0)
        run.move_nodes(w.params.t_del)
        run.update_mhd(w.params.t_del)
        run.init_seed_population(w.seed, w.perturb)
        runs.append(run)
    t = w.params.t_del
    for _ in range(6):
        for run in runs:
            run.move_nodes(w.params.t_del)
            run.update_mhd(t + w.params.t_del)
            run.update_energetic_particles(t)
        t += w.params.t_del
    st = runs[1].read_stats()
    j64, j32 = (run.omni_flux() for run in runs)
    for run in runs:
        run.close()
    assert st.max_substeps_stream > 300
    assert flux_err(j32, j64) <= FLUX_RTOL
