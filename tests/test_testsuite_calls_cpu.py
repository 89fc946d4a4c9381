"""The recorded testsuite calls (tests/golden/testsuite_*.npz) load and run
on the CPU restatement.  These are the inputs of hot-path calls that the
reference's own driver made during whole runs of its testsuite (the
restatement reproduces those runs' golden digests byte for byte,
test_testsuite_digest.py); test_gpu_testsuite_calls.py replays them on the
GPU.  Here: the fixtures are complete and consistent, and the restatement
runs each call without an error."""
import glob
import os

import numpy as np
import pytest

from eprem_gb300 import abi

from helpers import CALL_EP, CALL_MHD, load_call, oracle_call

FIXTURES = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "testsuite_*.npz")))


def test_fixtures_cover_every_kind_of_call():
    kinds = {int(np.load(p)["kind"][0]) for p in FIXTURES}
    assert kinds == {0, 1, 2, 3}, kinds
    assert {os.path.basename(p).split("_")[1] for p in FIXTURES} >= {"wind", "cone", "mas"}


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p)[10:-4] for p in FIXTURES])
def test_recorded_call_runs_on_the_oracle(path, oracle_lib):
    rec = load_call(path)
    d = rec["dims"]
    assert d.precision == abi.EPREM_FP64 and 1 <= d.num_streams <= 6
    if rec["kind"] == CALL_EP:
        assert rec["f"].size == d.num_streams * d.num_nodes * d.num_energies * d.num_mu
        assert np.all(np.isfinite(rec["f"])) and np.all(rec["f"] > 0)
    if rec["kind"] == CALL_MHD and "slots" in rec:
        assert rec["mas_on"]
    f, nodes, st = oracle_call(oracle_lib, rec)
    assert np.all(np.isfinite(nodes[abi.NODE["RMAG"]]))
    if f is not None:
        assert np.all(np.isfinite(f)) and st.max_substeps_stream >= 1
