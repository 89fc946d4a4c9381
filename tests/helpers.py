"""Shared helpers of the test suite: build a primed run state and run the
oracle or the GPU on it."""
import numpy as np

from eprem_gb300 import abi, workloads as W


def primed_state(w, orc, precision=abi.EPREM_FP64):
    """Positions on Parker spirals, analytic MHD after one node push
    (updateMhd, moveNodes, updateMhd as the driver does, src/eprem.c:620-639),
    and the perturbed seed distribution."""
    d = w.dims(precision)
    g = W.build_grids(w)
    nodes = W.initial_nodes(w)
    orc.update_mhd(d, w.params, nodes, 0.0)
    orc.move_nodes(d, w.params, nodes, w.params.t_del)
    orc.update_mhd(d, w.params, nodes, w.params.t_del)
    f = W.initial_f(w, nodes, g)
    return d, g, f, nodes


def oracle_update(orc, w, g, f, nodes, calls=1, nthreads=8):
    f = f.copy()
    nodes = nodes.copy()
    gs, keep = W.grids_struct(g)
    stats = []
    for _ in range(calls):
        rc, st, err = orc.update_energetic_particles(w.dims(), w.params, gs, f, nodes,
                                                     nthreads=nthreads)
        assert rc == 0, err
        stats.append(st)
    return f, nodes, stats


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b) / np.abs(b)))


# ---- calls recorded from whole runs of the reference's testsuite ----------
# (tests/golden/make_testsuite_calls.py writes them; kinds as there)
CALL_EP, CALL_MHD, CALL_MOVE, CALL_MASMOVE = 0, 1, 2, 3


def load_call(path):
    """A recorded hot-path call: its kind, argument (t_global or dt),
    dimensions, parameters, grids, inputs and, for MAS calls, the MAS slots
    (abi structs whose arrays are kept alive in the returned dict)."""
    z = dict(np.load(path))
    rec = {"kind": int(z["kind"][0]), "arg": float(z["arg"][0])}
    rec["dims"] = abi.Dims.from_buffer_copy(z["dims"].tobytes())
    rec["params"] = abi.Params.from_buffer_copy(z["params"].tobytes())
    rec["grids"] = {k: z[k] for k in ("egrid", "vgrid", "vgrid_i", "mugrid", "rigidity")}
    rec["grids"]["dlnp"] = float(z["dlnp"][0])
    rec["grids"]["dmu"] = float(z["dmu"][0])
    d = rec["dims"]
    sn = d.num_streams * d.num_nodes
    rec["nodes"] = z["nodes"].reshape(abi.NODE_NFIELDS, sn).copy()
    if "f" in z:
        rec["f"] = z["f"].copy()
    rec["mas_on"] = bool(z["mas_on"][0])
    if "mas_params" in z:
        rec["mas_params"] = abi.MasParams.from_buffer_copy(z["mas_params"].tobytes())
        rec["s_cor"] = float(z["s_cor"][0])
        rec["phi_offset"] = float(z["phi_offset"][0])
        keep, slots = [], []
        for s in range(2):
            sl = abi.MasSlice()
            dims = z[f"slot{s}_dims"].reshape(abi.MAS_NFIELDS, 3)
            for fld in range(abi.MAS_NFIELDS):
                for a in range(3):
                    sl.dims[fld][a] = int(dims[fld, a])
                    m = np.ascontiguousarray(z[f"slot{s}_mesh{fld}_{a}"], dtype=np.float32)
                    keep.append(m)
                    sl.mesh[fld][a] = m.ctypes.data_as(abi.C.POINTER(abi.C.c_float))
                data = np.ascontiguousarray(z[f"slot{s}_data{fld}"], dtype=np.float32)
                keep.append(data)
                sl.data[fld] = data.ctypes.data_as(abi.C.POINTER(abi.C.c_float))
            slots.append(sl)
        rec["slots"], rec["_keep"] = slots, keep
    return rec


def oracle_call(orc, rec):
    """Run the recorded call on the CPU restatement: (f, nodes, stats)."""
    import ctypes as C
    import oracle as O
    d, p = rec["dims"], rec["params"]
    f = rec["f"].copy() if "f" in rec else None
    nodes = rec["nodes"].copy()
    st = None
    if rec["kind"] == CALL_EP:
        gs, keep = W.grids_struct(rec["grids"])
        rc, st, err = orc.update_energetic_particles(d, p, gs, f, nodes, nthreads=8)
        assert rc == 0, err
    elif rec["kind"] == CALL_MOVE:
        assert orc.move_nodes(d, p, nodes, rec["arg"]) == 0
    else:
        mas = None
        if "slots" in rec:
            mas = O.MasState(C.pointer(rec["slots"][0]), C.pointer(rec["slots"][1]),
                             rec["s_cor"], rec["phi_offset"], rec["mas_params"])
        if rec["kind"] == CALL_MHD and not rec["mas_on"]:
            assert orc.update_mhd(d, p, nodes, rec["arg"]) == 0
        elif rec["kind"] == CALL_MHD:
            assert orc.mas_update_mhd(d, p, nodes, mas, rec["arg"]) == 0
        else:
            assert orc.mas_move_nodes(d, p, nodes, mas, rec["arg"]) == 0
    return f, nodes, st
