"""Golden record of a whole run of the CPU-runnable plain-method workload,
made once with the oracle (the CPU restatement, itself pinned bit for bit to
the reference's C) and committed as tests/golden/small_run_24h.npz.

Workload: 24 streams x 400 nodes (0.05-5 AU, log-spaced) x 20 energies
(0.1-100 MeV) x 20 mu, the analytic Parker wind of 400 km/s with |B| = 5 nT
and n = 5 cm^-3 at 1 AU, lambda_par = 0.3 AU at 1 GV scaling as R^(1/3),
power-law seed of index -3.5 with a 1% splitmix64(12345) perturbation; the
driver's 24 h: 96 steps of tDel = 0.0104167 d, each moveNodes + updateMhd +
updateEnergeticParticles with 30 EP sub-steps (src/eprem.c:620-671).

Stored: every step's log statistics (sub-cycle maxima, min tau and the cell
x sub-cycle counts), the final f of stream 0 in full, and per-(stream, node)
and per-(stream, energy, mu) sums of the final f (every stream checked).

Run from the repository root:  python tests/golden/make_small_run.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

import oracle as O  # noqa: E402
from eprem_gb300 import workloads as W  # noqa: E402
from helpers import primed_state  # noqa: E402

STEPS = 96
OUT = os.path.join(ROOT, "tests", "golden", "small_run_24h.npz")
STAT_FIELDS = ("max_subcycles_focusing", "max_subcycles_change", "max_substeps_stream",
               "min_tau", "stream_cell_subcycles", "focus_cell_subcycles",
               "change_cell_subcycles")


def main():
    O.build()
    o = O.Oracle()
    w = W.small_plain()
    d, g, f, nodes = primed_state(w, o)
    gs, keep = W.grids_struct(g)
    dt = w.params.t_del
    t = dt
    stats = np.zeros((STEPS, len(STAT_FIELDS)))
    for k in range(STEPS):
        assert o.move_nodes(d, w.params, nodes, dt) == 0
        assert o.update_mhd(d, w.params, nodes, t + dt) == 0
        rc, st, err = o.update_energetic_particles(d, w.params, gs, f, nodes,
                                                   nthreads=os.cpu_count() or 8)
        assert rc == 0, err
        stats[k] = [getattr(st, n) for n in STAT_FIELDS]
        t += dt
    S, N, E, M = d.num_streams, d.num_nodes, d.num_energies, d.num_mu
    f4 = f.reshape(S, N, E, M)
    np.savez_compressed(OUT, stats=stats, stat_fields=np.array(STAT_FIELDS),
                        f_stream0=f4[0].copy(), sum_sn=f4.sum(axis=(2, 3)),
                        sum_sem=f4.sum(axis=1), t_end=np.array([t]))
    print(f"wrote {OUT}: {os.path.getsize(OUT)} bytes; last step stats {stats[-1]}")


if __name__ == "__main__":
    main()
