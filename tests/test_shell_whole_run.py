"""Whole runs with shell diffusion on: the reference's own driver and sources
(oracle/_ref/eprem_ref) against the same driver over the drop-in and the CPU
restatement (oracle/_ref/eprem_oracle_dropin), on the testsuite's `wind`
configuration (and `cone`, with the ideal shock, when EPREM_SLOW_TESTS is set)
switched to useShellDiffusion=1, kperxkpar=0.05.  The testsuite has no golden
for shell diffusion, so the reference's run is the golden here: the observer
output digest and the log must be identical, and must differ from the
testsuite's diffusion-off golden (the coupling is not a no-op).  This pins
the drop-in's NEWS hand-over (taken from the grid's links after
gridStructInit) and the restatement's sub-step order on whole runs.
"""
import concurrent.futures as cf
import os
import re
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle as _orc  # noqa: E402  (the reference tree's location only)

REF = _orc.reference_root() or ""

pytestmark = pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "testsuite")),
                                reason="reference source tree not present")

CASES = ["wind"] + (["cone"] if os.environ.get("EPREM_SLOW_TESTS") else [])
EXES = ["eprem_ref", "eprem_oracle_dropin"]


@pytest.fixture(scope="module")
def runs(tmp_path_factory):
    subprocess.check_call(["make", "-s", "-j8", "-C", os.path.join(ROOT, "oracle"), "ref",
                           "ref-dropin", f"REF={REF}"])
    base = tmp_path_factory.mktemp("shell_runs")

    def run(key):
        exe, case = key
        top = base / f"{exe}_{case}"
        d = top / "run"
        d.mkdir(parents=True)
        os.symlink(os.path.join(REF, "testsuite", case, "input"), top / "input")
        text = open(os.path.join(REF, "testsuite", case, "input", "eprem_input_file")).read()
        text, n1 = re.subn(r"(?m)^useShellDiffusion=0", "useShellDiffusion=1", text)
        text, n2 = re.subn(r"(?m)^kperxkpar=0\.01", "kperxkpar=0.05", text)
        assert n1 == n2 == 1
        (d / "eprem_input_file").write_text(text)
        env = dict(os.environ, EPREM_ORACLE_THREADS="4")
        with open(d / "eprem.log", "w") as lo, open(d / "eprem.err", "w") as le:
            rc = subprocess.call([os.path.join(ROOT, "oracle", "_ref", exe), "eprem_input_file"],
                                 cwd=d, stdout=lo, stderr=le, env=env, timeout=900)
        return key, str(d), rc

    keys = [(e, c) for c in CASES for e in EXES]
    with cf.ThreadPoolExecutor(max_workers=len(keys)) as ex:
        res = list(ex.map(run, keys))
    for key, d, rc in res:
        assert rc == 0, f"{key} exited {rc}: {open(os.path.join(d, 'eprem.err')).read()[-2000:]}"
    return {key: d for key, d, _ in res}


def _log(path):
    skip = re.compile(r"Compute time for step|Run started|Run finished|Run real time|"
                      r"Run data time|^Processors:|seconds|[Tt]imer")
    return [ln.rstrip() for ln in open(path).read().splitlines() if not skip.search(ln)]


@pytest.mark.parametrize("case", CASES)
def test_dropin_run_identical_to_reference_run(runs, case):
    import digest as D
    ref = D.digest_run(runs[("eprem_ref", case)])
    got = D.digest_run(runs[("eprem_oracle_dropin", case)])
    if got != ref:
        a, b = D.parse_digest(got), D.parse_digest(ref)
        bad = [k for k in b if a.get(k) != b[k]]
        pytest.fail(f"{len(bad)} of {len(b)} digest entries differ, first: {bad[:3]}")
    off = open(os.path.join(REF, "testsuite", case, "reference", "eprem_digest.txt")).read()
    assert ref != off
    la = _log(os.path.join(runs[("eprem_ref", case)], "eprem.log"))
    lb = _log(os.path.join(runs[("eprem_oracle_dropin", case)], "eprem.log"))
    assert sum(ln.startswith("Step:") or "Maximum subcycles" in ln for ln in la) > 0
    assert la == lb
