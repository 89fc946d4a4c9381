"""Whole runs with drift on: the reference's own driver and sources
(oracle/_ref/eprem_ref) against the same driver over the drop-in and the CPU
restatement (oracle/_ref/eprem_oracle_dropin), on the testsuite's `wind`
configuration switched to useDrift=1 -- alone, and with shell diffusion
(kperxkpar = 0.05) -- and `cone` (ideal shock) with drift when
EPREM_SLOW_TESTS is set.  The testsuite has no golden with drift, so the
reference's run is the golden: observer digest and log identical, and both
different from the testsuite's drift-off golden.  This pins the drop-in's
drift hand-over (curl(B)/B^2 formed by updateMhd from the first call, the
NEWS links from the first particle update) and the restatement's
DriftShellData on whole runs."""
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

VARIANTS = [("wind", False), ("wind", True)] + (
    [("cone", False)] if os.environ.get("EPREM_SLOW_TESTS") else [])
EXES = ["eprem_ref", "eprem_oracle_dropin"]


def drift_config(case, shell):
    text = open(os.path.join(REF, "testsuite", case, "input", "eprem_input_file")).read()
    text, n = re.subn(r"(?m)^useDrift=0", "useDrift=1", text)
    assert n == 1
    if shell:
        text, n1 = re.subn(r"(?m)^useShellDiffusion=0", "useShellDiffusion=1", text)
        text, n2 = re.subn(r"(?m)^kperxkpar=0\.01", "kperxkpar=0.05", text)
        assert n1 == n2 == 1
    return text


@pytest.fixture(scope="module")
def runs(tmp_path_factory):
    subprocess.check_call(["make", "-s", "-j8", "-C", os.path.join(ROOT, "oracle"), "ref",
                           "ref-dropin", f"REF={REF}"])
    base = tmp_path_factory.mktemp("drift_runs")

    def run(key):
        exe, case, shell = key
        top = base / f"{exe}_{case}_{int(shell)}"
        d = top / "run"
        d.mkdir(parents=True)
        os.symlink(os.path.join(REF, "testsuite", case, "input"), top / "input")
        (d / "eprem_input_file").write_text(drift_config(case, shell))
        env = dict(os.environ, EPREM_ORACLE_THREADS="4")
        with open(d / "eprem.log", "w") as lo, open(d / "eprem.err", "w") as le:
            rc = subprocess.call([os.path.join(ROOT, "oracle", "_ref", exe), "eprem_input_file"],
                                 cwd=d, stdout=lo, stderr=le, env=env, timeout=900)
        return key, str(d), rc

    keys = [(e, c, sh) for c, sh in VARIANTS for e in EXES]
    with cf.ThreadPoolExecutor(max_workers=len(keys)) as ex:
        res = list(ex.map(run, keys))
    for key, d, rc in res:
        assert rc == 0, f"{key} exited {rc}: {open(os.path.join(d, 'eprem.err')).read()[-2000:]}"
    return {key: d for key, d, _ in res}


def _log(path):
    skip = re.compile(r"Compute time for step|Run started|Run finished|Run real time|"
                      r"Run data time|^Processors:|seconds|[Tt]imer")
    return [ln.rstrip() for ln in open(path).read().splitlines() if not skip.search(ln)]


@pytest.mark.parametrize("case,shell", VARIANTS, ids=[f"{c}{'+shell' if s else ''}"
                                                      for c, s in VARIANTS])
def test_drift_run_identical_to_reference_run(runs, case, shell):
    import digest as D
    ref = D.digest_run(runs[("eprem_ref", case, shell)])
    got = D.digest_run(runs[("eprem_oracle_dropin", case, shell)])
    if got != ref:
        a, b = D.parse_digest(got), D.parse_digest(ref)
        bad = [k for k in b if a.get(k) != b[k]]
        pytest.fail(f"{len(bad)} of {len(b)} digest entries differ, first: {bad[:3]}")
    off = open(os.path.join(REF, "testsuite", case, "reference", "eprem_digest.txt")).read()
    assert ref != off
    la = _log(os.path.join(runs[("eprem_ref", case, shell)], "eprem.log"))
    lb = _log(os.path.join(runs[("eprem_oracle_dropin", case, shell)], "eprem.log"))
    assert la == lb
