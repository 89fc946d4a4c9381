"""Generate the committed golden vectors from the reference's own C.

Each case runs entirely inside the reference (oracle/_ref/libeprem_ref.so,
built from the reference source tree by oracle/Makefile): node positions are
loaded into its `grid`, its updateMhd / moveNodes / updateMhd prime the MHD
fields as its driver does (src/eprem.c:620-639), and its
updateEnergeticParticles advances f.  Inputs and outputs are stored so the
tests can check the oracle against the reference where the reference tree is
absent.

Run from the repository root:  python tests/golden/make_golden.py [case ...]
(needs the reference tree, oracle.reference_root(); each case runs in a fresh process because the
reference allocates its globals once per process).
"""
import ctypes as C
import multiprocessing as mp
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def cases():
    from eprem_gb300 import workloads as W
    return {
        "wind_like": W.testsuite_like("wind", 1, 1, 20),
        "cone_like_shock": W.testsuite_like("cone", 1, 1, 24),
        "plain_alg3": W.custom(1, 1, 16, 8, 8, num_ep_steps=3, adiabatic_focus_alg=3,
                               adiabatic_change_alg=3),
        "plain_alg2_mfpB_damped": W.custom(1, 1, 16, 8, 8, num_ep_steps=3, adiabatic_focus_alg=2,
                                           adiabatic_change_alg=2, mfp_type=2, damp_cooling=0.4),
        "seed_only": W.custom(1, 1, 16, 8, 6, num_ep_steps=2, use_parallel_diffusion=0,
                              use_adiabatic_focus=0, use_adiabatic_change=0),
        # shell diffusion (DiffuseShellData) on the reference's own NEWS links:
        # a weak coupling and one strong enough that most hand-overs hit the
        # 0.025 cap
        "shell_2x2_weak": W.custom(2, 2, 16, 8, 6, num_ep_steps=3),
        "shell_3x2_capped": W.custom(3, 2, 12, 6, 6, num_ep_steps=2),
    }


# kperxkpar of the shell-diffusion cases
SHELL = {"shell_2x2_weak": 0.01, "shell_3x2_capped": 50.0}


def run_case(name, q):
    import oracle as O
    from eprem_gb300 import abi, workloads as W
    w = cases()[name]
    ref = O.Reference()
    g = ref.setup(w)
    extra = {}
    if name in SHELL:  # before ref.load: the NEWS set-up also places nodes
        extra = dict(news=ref.shell_diffusion(SHELL[name], w.dims().num_streams),
                     kperxkpar=np.array([SHELL[name]]))
    nodes0 = W.initial_nodes(w)
    f0 = np.zeros(w.cells)
    ref.load(f0, nodes0)
    ref.update_mhd(0.0)
    ref.move_nodes(w.params.t_del)
    ref.update_mhd(w.params.t_del)
    nodes_in = np.zeros_like(nodes0)
    ref.store(f0, nodes_in)
    f_in = W.initial_f(w, nodes_in, g)
    ref.load(f_in, nodes_in)
    rc, st = ref.update_energetic_particles(0.0)
    f_out = np.zeros_like(f_in)
    nodes_out = np.zeros_like(nodes_in)
    ref.store(f_out, nodes_out)
    q.put(dict(name=name, rc=rc, nodes0=nodes0, nodes_in=nodes_in, f_in=f_in, f_out=f_out,
               nodes_out=nodes_out,
               stats=np.array([st.max_subcycles_change, st.max_subcycles_focusing, st.min_tau]),
               dims=np.frombuffer(bytes(w.dims()), dtype=np.uint8),
               params=np.frombuffer(bytes(w.params), dtype=np.uint8),
               grids=np.concatenate([g["egrid"], g["vgrid"], g["vgrid_i"], g["rigidity"],
                                     g["mugrid"], [g["dlnp"], g["dmu"]]]), **extra))


def main(names=None):
    ctx = mp.get_context("spawn")
    for name in names or cases():
        q = ctx.Queue()
        p = ctx.Process(target=run_case, args=(name, q))
        p.start()
        out = q.get()
        p.join()
        assert out["rc"] == 0, name
        del out["name"], out["rc"]
        path = os.path.join(HERE, f"ref_{name}.npz")
        np.savez_compressed(path, **out)
        print(path, os.path.getsize(path))


if __name__ == "__main__":
    main(sys.argv[1:])
