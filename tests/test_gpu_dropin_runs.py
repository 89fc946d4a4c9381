"""The drop-in on the GPU: whole runs of the reference's own driver
(src/eprem.c, unchanged) with updateEnergeticParticles, updateMhd, moveNodes,
masMoveNodes, rotSunAndSpawnShell and the dataDumpIO / initEnergeticParticles
wrappers resolved to eprem_gb300/host/eprem_dropin.c over libeprem_gpu.so
(eprem_gb300/host/Makefile `link`), on the reference's testsuite cases seed,
wind and cone (ideal shock), FP64 form.  Each run is checked against
  * the testsuite's golden digest (testsuite/<case>/reference/eprem_digest.txt):
    shape and the 6-significant-figure min / max / mean / sum / rms of every
    variable of every observer file -- the SHA-256 lines need bit equality,
    which the GPU's fused multiply-adds do not keep;
  * the golden eprem.log: every step's sub-cycle maxima and minimum tau
    (wall-clock lines and the rank count left out);
  * the same driver over the CPU restatement (oracle/_ref/eprem_oracle_dropin,
    whose digests are the goldens byte for byte): every captured observer
    array within 1e-12 relative (1e-10 of its scale for the background
    fields, which pass through the node push and the MAS-free analytic wind).
The reference tree comes from oracle.reference_root() (the staged copy travels
with the working copy); without it these tests are skipped.
"""
import os
import re
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle as _orc  # noqa: E402  (the reference tree's location and the checker)

REF = _orc.reference_root() or ""

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "testsuite")),
                                 reason="reference source tree not present")]

CASES = ["seed", "wind", "cone"]
GPU_EXE = os.path.join(ROOT, "eprem_gb300", "host", "_link", "eprem_gb300")
ORC_EXE = os.path.join(ROOT, "oracle", "_ref", "eprem_oracle_dropin")


@pytest.fixture(scope="module")
def runs(tmp_path_factory):
    from eprem_gb300 import build
    build.build()
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "eprem_gb300", "host"), "link",
                           f"REF={REF}"])
    subprocess.check_call(["make", "-s", "-j8", "-C", os.path.join(ROOT, "oracle"), "ref-dropin",
                           f"REF={REF}"])
    base = tmp_path_factory.mktemp("dropin_gpu")
    out = {}
    for case in CASES:
        for tag, exe in (("gpu", GPU_EXE), ("oracle", ORC_EXE)):
            top = base / f"{tag}_{case}"
            d = top / "run"
            d.mkdir(parents=True)
            os.symlink(os.path.join(REF, "testsuite", case, "input"), top / "input")
            (d / "eprem_input_file").write_text(
                open(os.path.join(REF, "testsuite", case, "input", "eprem_input_file")).read())
            env = dict(os.environ, EPREM_ORACLE_THREADS="8")
            env.pop("EPREM_GPU_FP32", None)
            with open(d / "eprem.log", "w") as lo, open(d / "eprem.err", "w") as le:
                rc = subprocess.call([exe, "eprem_input_file"], cwd=d, stdout=lo, stderr=le,
                                     env=env, timeout=900)
            assert rc == 0, f"{tag} {case} exited {rc}: {open(d / 'eprem.err').read()[-2000:]}"
            out[(tag, case)] = str(d)
    return out


def _log(path):
    skip = re.compile(r"Compute time for step|Run started|Run finished|Run real time|"
                      r"Run data time|^Processors:|seconds|[Tt]imer")
    return [ln.rstrip() for ln in open(path).read().splitlines() if not skip.search(ln)]


@pytest.mark.parametrize("case", CASES)
def test_gpu_run_digest_statistics_equal_golden(runs, case):
    import digest as D
    got = D.parse_digest(D.digest_run(runs[("gpu", case)]))
    want = D.parse_digest(open(os.path.join(REF, "testsuite", case, "reference",
                                            "eprem_digest.txt")).read())
    assert set(got) == set(want)
    bad = [k for k in want if (got[k]["shape"], got[k]["stats"]) != (want[k]["shape"],
                                                                      want[k]["stats"])]
    assert not bad, f"{len(bad)} of {len(want)} variables differ, first: {bad[:3]} " \
                    f"{[(got[k]['stats'], want[k]['stats']) for k in bad[:2]]}"


@pytest.mark.parametrize("case", CASES)
def test_gpu_run_log_equals_golden(runs, case):
    got = _log(os.path.join(runs[("gpu", case)], "eprem.log"))
    want = _log(os.path.join(REF, "testsuite", case, "reference", "eprem.log"))
    assert got == want, next(((i, a, b) for i, (a, b) in enumerate(zip(want, got)) if a != b),
                             (len(want), len(got)))


@pytest.mark.parametrize("case", CASES)
def test_gpu_run_arrays_match_oracle_run(runs, case):
    import glob
    import digest as D
    caps = sorted(glob.glob(os.path.join(runs[("oracle", case)], "obs*.nc.cap")))
    assert caps
    worst = {}
    for cap in caps:
        ref = D.read_capture(cap)
        got = D.read_capture(os.path.join(runs[("gpu", case)], os.path.basename(cap)))
        assert set(ref) == set(got)
        for name, (a, sc, off) in ref.items():
            b = got[name][0]
            a64 = np.asarray(D.unpacked(a, sc, off), dtype=np.float64)
            b64 = np.asarray(D.unpacked(b, sc, off), dtype=np.float64)
            assert a64.shape == b64.shape, name
            if name == "Dist":
                nz = a64 != 0
                err = float(np.max(np.abs(b64[nz] - a64[nz]) / np.abs(a64[nz]), initial=0.0))
                tol = 1e-12
            else:
                scale = max(float(np.max(np.abs(a64), initial=0.0)), 1e-300)
                err = float(np.max(np.abs(b64 - a64), initial=0.0)) / scale
                tol = 1e-10
            worst[name] = max(worst.get(name, 0.0), err)
            assert err <= tol, (os.path.basename(cap), name, err)
    assert "Dist" in worst


def test_gpu_flux_output_run_matches_reference(tmp_path):
    """streamFluxOutput on the GPU: dataDumpIO brings down the device's flux
    (S*N*E values) instead of f; the flux files of the testsuite's wind case
    (streamFluxOutput=1, domain dump off) within 1e-12 of the reference's
    own run, every other variable within 1e-10."""
    from test_flux_output_run import compare_flux_runs, flux_config, run_case
    subprocess.check_call(["make", "-s", "-j8", "-C", os.path.join(ROOT, "oracle"), "ref",
                           f"REF={REF}"])
    from eprem_gb300 import build
    build.build()
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "eprem_gb300", "host"), "link",
                           f"REF={REF}"])
    text = flux_config()
    ref = run_case(os.path.join(ROOT, "oracle", "_ref", "eprem_ref"), "wind", tmp_path, text)
    gpu = run_case(GPU_EXE, "wind", tmp_path, text)
    assert compare_flux_runs(gpu, ref, 1e-12) > 0.0


def test_gpu_drift_run_matches_oracle_run(tmp_path):
    """useDrift through the drop-in on the GPU: the testsuite's wind case
    with useDrift=1, every observer array within 1e-12 of the same driver
    over the CPU restatement (whose run is byte-identical to the
    reference's own, test_drift_whole_run.py)."""
    from test_drift_whole_run import drift_config
    from test_flux_output_run import run_case
    subprocess.check_call(["make", "-s", "-j8", "-C", os.path.join(ROOT, "oracle"), "ref-dropin",
                           f"REF={REF}"])
    from eprem_gb300 import build
    build.build()
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "eprem_gb300", "host"), "link",
                           f"REF={REF}"])
    text = drift_config("wind", False)
    orc = run_case(ORC_EXE, "wind", tmp_path, text, {"EPREM_ORACLE_THREADS": "8"})
    gpu = run_case(GPU_EXE, "wind", tmp_path, text)
    import glob
    import digest as D
    caps = sorted(glob.glob(os.path.join(orc, "obs*.nc.cap")))
    assert caps
    for cap in caps:
        ref = D.read_capture(cap)
        got = D.read_capture(os.path.join(gpu, os.path.basename(cap)))
        for name, (a, sc, off) in ref.items():
            b = got[name][0]
            a64 = np.asarray(D.unpacked(a, sc, off), dtype=np.float64)
            b64 = np.asarray(D.unpacked(b, sc, off), dtype=np.float64)
            if name == "Dist":
                nz = a64 != 0
                err = float(np.max(np.abs(b64[nz] - a64[nz]) / np.abs(a64[nz]), initial=0.0))
                assert err <= 1e-12, (os.path.basename(cap), err)
            else:
                scale = max(float(np.max(np.abs(a64), initial=0.0)), 1e-300)
                assert float(np.max(np.abs(b64 - a64), initial=0.0)) / scale <= 1e-10, name
