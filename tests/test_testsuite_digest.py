"""Whole runs of the reference's own testsuite, checked against its goldens.

The reference's testsuite (testsuite/run_test_suite.sh in the reference) runs
the EPREM driver on five configurations -- `seed`, `wind`, `cone` (ideal
shock), `mas_wind` and `mas_cme` (MAS-coupled, HDF5 slice input) -- and passes
a case when the text digest of its observer output is identical to the stored
testsuite/<case>/reference/eprem_digest.txt (SHA-256 of every variable plus
6-significant-figure statistics); its eprem.log records the per-step
sub-cycle maxima and minimum tau.

Two binaries are run on each case (oracle/Makefile, reference tree needed):
  * eprem_ref: the reference's unchanged driver and sources with the one-rank
    MPI, config reader, netCDF capture and HDF5 reader of oracle/ref_shims.c
    -- shows the harness reproduces the goldens (they were made with 6 MPI
    ranks);
  * eprem_oracle_dropin: the same driver with updateEnergeticParticles,
    updateMhd, moveNodes and masMoveNodes resolved to
    eprem_gb300/host/eprem_dropin.c over the CPU restatement -- pins the
    restatement and the drop-in's handling of the reference globals on whole
    runs (shell spawning, the ideal shock, MAS slices and SetDT's time-step
    changes, output), bit for bit.
The reference's own runs of `cone` and `mas_wind` (2.5 and 3 minutes) run
when EPREM_SLOW_TESTS is set; every drop-in run always runs.
"""
import concurrent.futures as cf
import os
import re
import shutil
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle as _orc  # noqa: E402  (the reference tree's location only)

REF = _orc.reference_root() or ""

pytestmark = pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "testsuite")),
                                reason="reference source tree not present")

CASES = ["seed", "wind", "cone", "mas_wind", "mas_cme"]
SLOW_REF = {"cone", "mas_wind"}
SLOW = bool(os.environ.get("EPREM_SLOW_TESTS"))


def _runs():
    out = [("eprem_oracle_dropin", c) for c in CASES]
    out += [("eprem_ref", c) for c in CASES if c not in SLOW_REF or SLOW]
    return out


@pytest.fixture(scope="module")
def testsuite_runs(tmp_path_factory):
    """Run every (binary, case) once, in parallel processes; {key: rundir}."""
    subprocess.check_call(["make", "-s", "-j8", "-C", os.path.join(ROOT, "oracle"), "ref",
                           "ref-dropin", f"REF={REF}"])
    base = tmp_path_factory.mktemp("testsuite")

    def run(key):
        exe, case = key
        # the testsuite's layout: <case>/run holds the config, MAS inputs are
        # read from ../input/data/
        top = base / f"{exe}_{case}"
        d = top / "run"
        d.mkdir(parents=True)
        os.symlink(os.path.join(REF, "testsuite", case, "input"), top / "input")
        shutil.copy(os.path.join(REF, "testsuite", case, "input", "eprem_input_file"), d)
        env = dict(os.environ, EPREM_ORACLE_THREADS="4")
        with open(d / "eprem.log", "w") as lo, open(d / "eprem.err", "w") as le:
            rc = subprocess.call([os.path.join(ROOT, "oracle", "_ref", exe), "eprem_input_file"],
                                 cwd=d, stdout=lo, stderr=le, env=env, timeout=900)
        return key, str(d), rc

    with cf.ThreadPoolExecutor(max_workers=len(_runs())) as ex:
        res = list(ex.map(run, _runs()))
    for key, d, rc in res:
        assert rc == 0, f"{key} exited {rc}: {open(os.path.join(d, 'eprem.err')).read()[-2000:]}"
    return {key: d for key, d, _ in res}


def _params(key):
    exe, case = key
    marks = [] if (exe != "eprem_ref" or case not in SLOW_REF or SLOW) else [
        pytest.mark.skip(reason="set EPREM_SLOW_TESTS for the reference's own run of this case")]
    return pytest.param(exe, case, marks=marks, id=f"{exe}-{case}")


ALL = [_params((e, c)) for e in ("eprem_oracle_dropin", "eprem_ref") for c in CASES]


@pytest.mark.parametrize("exe,case", ALL)
def test_digest_identical_to_golden(testsuite_runs, exe, case):
    import digest as D
    got = D.digest_run(testsuite_runs[(exe, case)])
    want = open(os.path.join(REF, "testsuite", case, "reference", "eprem_digest.txt")).read()
    if got != want:
        a, b = D.parse_digest(got), D.parse_digest(want)
        bad = [k for k in b if a.get(k) != b[k]]
        pytest.fail(f"{len(bad)} of {len(b)} digest entries differ, first: {bad[:3]}")


def _log_lines(text):
    """The golden log without wall-clock lines and the MPI rank count."""
    skip = re.compile(r"Compute time for step|Run started|Run finished|Run real time|"
                      r"Run data time|^Processors:|seconds|[Tt]imer")
    return [ln.rstrip() for ln in text.splitlines() if not skip.search(ln)]


@pytest.mark.parametrize("exe,case", ALL)
def test_log_identical_to_golden(testsuite_runs, exe, case):
    got = _log_lines(open(os.path.join(testsuite_runs[(exe, case)], "eprem.log")).read())
    want = _log_lines(open(os.path.join(REF, "testsuite", case, "reference", "eprem.log")).read())
    steps = sum(1 for ln in want if ln.startswith("Step:") or "Maximum subcycles" in ln)
    assert steps > 0
    assert got == want, next(((i, a, b) for i, (a, b) in enumerate(zip(want, got)) if a != b),
                             (len(want), len(got)))
