"""Make the testsuite-call fixtures (tests/golden/testsuite_*.npz).

Each fixture holds the inputs of one call the reference's unchanged driver
made to the hot path during a whole run of one of the reference's testsuite
cases: dimensions, parameters, grids, f, every node field and, in MAS runs,
the two MAS slots.  tests/test_gpu_testsuite_calls.py replays each call
through the GPU library and compares it with the CPU restatement run on the
same inputs; the restatement reproduces these runs' golden digests byte for
byte (tests/test_testsuite_digest.py), so the GPU is checked on the states of
the testsuite's own trajectories (thinned streams after shell spawning, the
ideal shock, MAS slices), not only on synthetic ones.

The calls are recorded by the driver linked over the drop-in and the
restatement (oracle/_ref/eprem_oracle_dropin, oracle/abi_oracle.c), which
needs the reference source tree: run this in the build container,
    python tests/golden/make_testsuite_calls.py
Recorded (call index in the run's order of hot-path calls):
  wind      the last EP update, updateMhd and moveNodes;
  cone      the EP update half way through the run (the shock is out in the
            grid), the last updateMhd and moveNodes;
  mas_wind  the EP update half way through, the last updateMhd (MAS
            background) and masMoveNodes (RK4 through the MAS velocity);
  mas_cme   the last EP update.
Streams are independent on this path (no drift, no shell diffusion), so each
fixture keeps every k-th stream (at most 6) to stay small; the MAS slots are
kept only for the calls that read them.
"""
import os
import shutil
import struct
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.dirname(
    os.path.abspath(__file__)))), "oracle"))
import oracle as _orc  # noqa: E402  (the reference tree's location only)

REF = _orc.reference_root() or ""
EXE = os.path.join(ROOT, "oracle", "_ref", "eprem_oracle_dropin")
KINDS = {0: "ep", 1: "mhd", 2: "move", 3: "masmove"}
PLAN = {"wind": ("ep_last", "mhd_last", "move_last"),
        "cone": ("ep_mid", "mhd_last", "move_last"),
        "mas_wind": ("ep_mid", "mhd_last", "move_last"),
        "mas_cme": ("ep_last",)}
MAX_STREAMS = 6
_DT = {0: np.float64, 1: np.float32, 2: np.int32, 3: np.uint8}


def read_record(path):
    raw = open(path, "rb").read()
    out, pos = {}, 0
    while pos < len(raw):
        (nl,) = struct.unpack_from("<i", raw, pos)
        pos += 4
        name = raw[pos:pos + nl].decode()
        pos += nl
        t, n = struct.unpack_from("<iq", raw, pos)
        pos += 12
        dt = np.dtype(_DT[t])
        out[name] = np.frombuffer(raw, dtype=dt, count=n, offset=pos).copy()
        pos += n * dt.itemsize
    return out


def keep_streams(r):
    """Every k-th stream of the record, at most MAX_STREAMS of them."""
    sys.path.insert(0, ROOT)
    from eprem_gb300 import abi
    d = abi.Dims.from_buffer_copy(r["dims"].tobytes())
    S, N, E, M = d.num_streams, d.num_nodes, d.num_energies, d.num_mu
    step = -(-S // MAX_STREAMS)
    sel = np.arange(0, S, step)
    d.num_streams = len(sel)
    r["dims"] = np.frombuffer(bytes(d), dtype=np.uint8).copy()
    if "f" in r:
        r["f"] = r["f"].reshape(S, N * E * M)[sel].ravel()
    r["nodes"] = r["nodes"].reshape(-1, S, N)[:, sel, :].ravel()
    r["streams_kept"] = sel.astype(np.int32)
    if int(r["kind"][0]) == 0:  # EP updates do not read the MAS slots
        for k in [k for k in r if k.startswith("slot") or k in ("mas_params", "s_cor",
                                                                 "phi_offset")]:
            del r[k]
    return r


def run_case(case, workdir, env_extra):
    top = os.path.join(workdir, case)
    run = os.path.join(top, "run")
    os.makedirs(run, exist_ok=True)
    if not os.path.exists(os.path.join(top, "input")):
        os.symlink(os.path.join(REF, "testsuite", case, "input"), os.path.join(top, "input"))
    shutil.copy(os.path.join(REF, "testsuite", case, "input", "eprem_input_file"), run)
    env = dict(os.environ, EPREM_ORACLE_THREADS="8", **env_extra)
    subprocess.check_call([EXE, "eprem_input_file"], cwd=run, env=env,
                          stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)


def main():
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref-dropin",
                           f"REF={REF}"])
    for old in os.listdir(HERE):
        if old.startswith("testsuite_") and old.endswith(".npz"):
            os.remove(os.path.join(HERE, old))
    with tempfile.TemporaryDirectory() as work:
        for case, plan in PLAN.items():
            rec = os.path.join(work, case + "_rec")
            os.makedirs(rec)
            run_case(case, os.path.join(work, "a"), {"EPREM_ORACLE_RECORD": rec})
            calls = [ln.split() for ln in open(os.path.join(rec, "calls.txt"))]
            by_kind = {}
            for idx, kind, _ in calls:
                by_kind.setdefault(int(kind), []).append(int(idx))
            moves = sorted(by_kind.get(2, []) + by_kind.get(3, []))
            choice = {"ep_last": by_kind[0][-1], "ep_mid": by_kind[0][len(by_kind[0]) // 2],
                      "mhd_last": by_kind[1][-1], "move_last": moves[-1]}
            pick = [choice[p] for p in plan]
            os.remove(os.path.join(rec, "calls.txt"))
            run_case(case, os.path.join(work, "b"), {
                "EPREM_ORACLE_RECORD": rec,
                "EPREM_ORACLE_RECORD_AT": ",".join(str(i) for i in pick)})
            for i in pick:
                r = keep_streams(read_record(os.path.join(rec, f"call_{i}.rec")))
                name = f"testsuite_{case}_{KINDS[int(r['kind'][0])]}_{i}.npz"
                np.savez_compressed(os.path.join(HERE, name), **r)
                print(name, os.path.getsize(os.path.join(HERE, name)), "bytes")


if __name__ == "__main__":
    if not os.path.isdir(os.path.join(REF, "testsuite")):
        sys.exit("the reference source tree is needed to record the calls")
    main()
