"""streamFluxOutput through the drop-in: the observer files then hold the
omnidirectional flux (computeFlux, src/unifiedOutput.c:153-180) instead of
f, and the drop-in's dataDumpIO brings down the run's flux (S*N*E values)
instead of all of f, writing each row's mu-average J / (2E) into eParts for
the unchanged writer (eprem_gb300/host/eprem_dropin.c).  The testsuite's
`wind` case switched to streamFluxOutput=1 (epremDomain off: the domain dump
reads all of f) runs through the reference's own driver and sources
(oracle/_ref/eprem_ref) and through the same driver over the drop-in and the
CPU restatement (oracle/_ref/eprem_oracle_dropin): every flux value within
1e-14 relative (the mu-average passes through one division and back), every
other variable identical, and the digest statistics equal.
"""
import glob
import os
import re
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle as _orc  # noqa: E402  (the reference tree's location only)

REF = _orc.reference_root() or ""

pytestmark = pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "testsuite")),
                                reason="reference source tree not present")


def flux_config(case="wind"):
    """The testsuite case's configuration with streamFluxOutput on and the
    domain dump off."""
    text = open(os.path.join(REF, "testsuite", case, "input", "eprem_input_file")).read()
    text, n = re.subn(r"(?m)^epremDomain=1\s*$", "epremDomain=0", text)
    assert n == 1
    assert "streamFluxOutput" not in text
    return text + "\nstreamFluxOutput=1\n"


def run_case(exe, case, base, text, env=None):
    top = base / f"{os.path.basename(exe)}_{case}"
    d = top / "run"
    d.mkdir(parents=True)
    os.symlink(os.path.join(REF, "testsuite", case, "input"), top / "input")
    (d / "eprem_input_file").write_text(text)
    with open(d / "eprem.log", "w") as lo, open(d / "eprem.err", "w") as le:
        rc = subprocess.call([exe, "eprem_input_file"], cwd=d, stdout=lo, stderr=le,
                             env=dict(os.environ, **(env or {})), timeout=900)
    assert rc == 0, f"{exe} {case} exited {rc}: {open(d / 'eprem.err').read()[-2000:]}"
    return str(d)


def compare_flux_runs(got_dir, ref_dir, flux_rtol):
    import digest as D
    caps = sorted(glob.glob(os.path.join(ref_dir, "flux*.nc.cap")))
    assert caps, "no flux files written"
    assert not glob.glob(os.path.join(ref_dir, "obs*.nc.cap"))
    worst = 0.0
    for cap in caps:
        ref = D.read_capture(cap)
        got = D.read_capture(os.path.join(got_dir, os.path.basename(cap)))
        assert set(ref) == set(got)
        assert "flux" in ref
        for name, (a, sc, off) in ref.items():
            b = got[name][0]
            if name == "flux":
                nz = a != 0
                err = float(np.max(np.abs(b[nz] - a[nz]) / np.abs(a[nz]), initial=0.0))
                worst = max(worst, err)
                assert err <= flux_rtol, (os.path.basename(cap), err)
            else:
                yield_same = np.array_equal(a, b) or np.allclose(a, b, rtol=1e-10, atol=0.0)
                assert yield_same, (os.path.basename(cap), name)
    return worst


@pytest.fixture(scope="module")
def runs(tmp_path_factory):
    subprocess.check_call(["make", "-s", "-j8", "-C", os.path.join(ROOT, "oracle"), "ref",
                           "ref-dropin", f"REF={REF}"])
    base = tmp_path_factory.mktemp("flux_runs")
    text = flux_config()
    return {exe: run_case(os.path.join(ROOT, "oracle", "_ref", exe), "wind", base, text,
                          {"EPREM_ORACLE_THREADS": "4"})
            for exe in ("eprem_ref", "eprem_oracle_dropin")}


def test_dropin_flux_output_matches_reference(runs):
    import digest as D
    compare_flux_runs(runs["eprem_oracle_dropin"], runs["eprem_ref"], 1e-14)
    a = D.parse_digest(D.digest_run(runs["eprem_oracle_dropin"], "flux"))
    b = D.parse_digest(D.digest_run(runs["eprem_ref"], "flux"))
    assert set(a) == set(b) and len(b) > 0
    assert all(a[k]["stats"] == b[k]["stats"] for k in b)
