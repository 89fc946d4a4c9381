"""The GPU path on the states of the reference's own testsuite runs.

tests/golden/testsuite_*.npz hold the inputs of hot-path calls the
reference's unchanged driver made during whole runs of its testsuite cases
(wind, cone with the ideal shock, mas_wind and mas_cme with MAS slices),
recorded through the drop-in (tests/golden/make_testsuite_calls.py).  The CPU
restatement reproduces those runs' golden digests byte for byte
(test_testsuite_digest.py); here every recorded call runs through the GPU
library (C ABI, FP64 form, with the drop-in's upload / call / download
sequence) and through the restatement on the same inputs:
  * updateEnergeticParticles: f within 1e-12 relative, ds and the
    neighbouring |B| bit-equal, sub-cycle counts equal, min tau within 1e-13;
  * updateMhd (analytic with the ideal shock, or MAS) and moveNodes /
    masMoveNodes: every node field within 1e-10 of its scale (1e-13 for the
    plain fields of the analytic background), NaN / Inf in the same places.
The FP32 form runs the EP calls too.  These states hold f from 30 down to
1e-239: the seed spectrum's exponential cut-off puts up to 120 decades
between neighbouring energies, so one float exponent range (76 decades)
cannot hold a state, and the adiabatic change works on ln f, where a floored
neighbour in energy would move a cell far above the floor.  The FP32 form
keeps an exponent per (stream, node, energy) row; its omnidirectional flux
is held to 1e-3 of the FP64 flux over every (node, energy) with
J > 1e-30 max J, the metric's own mask.
"""
import glob
import os

import numpy as np
import pytest

from eprem_gb300 import EpremRun, abi

from helpers import CALL_EP, CALL_MASMOVE, CALL_MHD, CALL_MOVE, load_call, oracle_call, rel_err

pytestmark = pytest.mark.gpu

FIXTURES = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "testsuite_*.npz")))
IDS = [os.path.basename(p)[10:-4] for p in FIXTURES]


def _gpu_call(rec, precision=abi.EPREM_FP64):
    d = abi.Dims.from_buffer_copy(bytes(rec["dims"]))
    d.precision = precision
    run = EpremRun(d, rec["params"], rec["grids"])
    try:
        if "f" in rec:
            run.upload_f(rec["f"])
        run.upload_nodes(rec["nodes"])
        if "slots" in rec:
            run.mas_init(rec["mas_params"])
            run.mas_load_slice(0, rec["slots"][0])
            run.mas_load_slice(1, rec["slots"][1])
            run.mas_select(0, 1, rec["s_cor"], rec["phi_offset"])
            run.mas_use(rec["mas_on"])
        st = None
        if rec["kind"] == CALL_EP:
            run.update_energetic_particles(rec["arg"])
            st = run.read_stats()
        elif rec["kind"] == CALL_MHD:
            run.update_mhd(rec["arg"])
        elif rec["kind"] == CALL_MOVE:
            run.move_nodes(rec["arg"])
        else:
            run.mas_move_nodes(rec["arg"])
        f = run.download_f() if "f" in rec else None
        flux = run.omni_flux() if "f" in rec else None
        return f, run.download_nodes(), st, flux
    finally:
        run.close()


def _nodes_close(a, b, tol_plain):
    for name in abi.NODE_FIELDS:
        i = abi.NODE[name]
        same = (a[i] == b[i]) | (np.isnan(a[i]) & np.isnan(b[i]))
        assert np.array_equal(np.isfinite(a[i]), np.isfinite(b[i])), name
        fin = np.isfinite(b[i])
        scale = max(np.max(np.abs(b[i][fin]), initial=0.0), 1e-300)
        err = np.max(np.where(same, 0.0, np.abs(a[i] - b[i]))) / scale
        tol = 1e-10 if name in ("DLNB", "DLNN", "DUPAR", "DIVV") else tol_plain
        assert err <= tol, (name, err)


@pytest.mark.parametrize("path", FIXTURES, ids=IDS)
def test_recorded_call_matches_oracle(path, oracle_lib):
    rec = load_call(path)
    f_ref, nodes_ref, st_ref = oracle_call(oracle_lib, rec)
    f, nodes, st, _ = _gpu_call(rec)
    if rec["kind"] == CALL_EP:
        assert rel_err(f, f_ref) <= 1e-12
        for fld in ("DS", "BMAG_PLUS", "BMAG_MINUS"):
            np.testing.assert_array_equal(nodes[abi.NODE[fld]], nodes_ref[abi.NODE[fld]])
        assert st.max_subcycles_focusing == st_ref.max_subcycles_focusing
        assert st.max_subcycles_change == st_ref.max_subcycles_change
        assert st.max_substeps_stream == st_ref.max_substeps_stream
        assert st.stream_cell_subcycles == st_ref.stream_cell_subcycles
        assert abs(st.min_tau - st_ref.min_tau) <= 1e-13 * st_ref.min_tau
    else:
        mas = rec["kind"] == CALL_MASMOVE or (rec["kind"] == CALL_MHD and rec["mas_on"])
        _nodes_close(nodes, nodes_ref, 1e-10 if mas else 1e-13)


EP = [(p, i) for p, i in zip(FIXTURES, IDS) if "_ep_" in os.path.basename(p)]


@pytest.mark.parametrize("path", [p for p, _ in EP], ids=[i for _, i in EP])
def test_recorded_ep_call_fp32_flux(path, oracle_lib):
    rec = load_call(path)
    f_ref, _, _ = oracle_call(oracle_lib, rec)
    from eprem_gb300 import workloads as W
    gs, keep = W.grids_struct(rec["grids"])
    j_ref = oracle_lib.omni_flux(rec["dims"], gs, f_ref)
    _, _, _, j = _gpu_call(rec, abi.EPREM_FP32)
    mask = j_ref > 1e-30 * j_ref.max()
    assert np.max(np.abs(j[mask] - j_ref[mask]) / j_ref[mask]) <= 1e-3
