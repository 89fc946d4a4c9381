"""ctypes access to the oracle libraries -- TEST INFRASTRUCTURE ONLY.

* ``Oracle``    -> oracle/liboracle.so, the CPU restatement (eprem_oracle.c);
* ``Reference`` -> oracle/_ref/libeprem_ref.so, the reference's own C compiled
  from its source tree (only present where that tree exists), or
  oracle/_ref/native/libeprem_ref_native.so, the same compiled with the
  reference's own optimisation flags (the timed CPU baseline).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module, and only to check or time against it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from eprem_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libeprem_ref.so")
# the reference compiled with its own flags (-O3 -march=native), for timing
NATIVE_LIB = os.path.join(HERE, "_ref", "native", "libeprem_ref_native.so")
DP = C.POINTER(C.c_double)


STAGED = os.path.join(HERE, "_ref", "tree")


def reference_root() -> str | None:
    """The reference's source tree: $EPREM_REF, else the staged copy
    oracle/_ref/tree (oracle/Makefile `stage`), else None."""
    for cand in (os.environ.get("EPREM_REF"), STAGED):
        if cand and os.path.isdir(os.path.join(cand, "src")):
            return cand
    return None


def build(ref: bool = False) -> None:
    """Compile liboracle.so and, when asked and the reference tree is
    present, the reference harness (libeprem_ref.so), the reference's own
    driver (eprem_ref) and the driver over the drop-in and this restatement
    (eprem_oracle_dropin)."""
    subprocess.check_call(["make", "-s", "-C", HERE, "all"])
    if not ref:
        return
    if not os.environ.get("EPREM_REF"):
        subprocess.check_call(["make", "-s", "-C", HERE, "stage"])
    root = reference_root()
    if root:
        subprocess.check_call(["make", "-s", "-j8", "-C", HERE, "ref", "ref-dropin",
                               "ref-native", f"REF={root}"])


def _dp(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(DP)


class Oracle:
    def __init__(self, path: str = LIB):
        if not os.path.exists(path):
            build()
        lib = C.CDLL(path)
        lib.orc_update_energetic_particles_range.argtypes = [
            C.POINTER(abi.Dims), C.POINTER(abi.Params), C.POINTER(abi.Grids), DP, DP, C.c_int,
            C.c_int, C.POINTER(abi.EpStats), C.c_int, C.c_char_p]
        lib.orc_update_energetic_particles_range.restype = C.c_int
        lib.orc_update_energetic_particles_news.argtypes = [
            C.POINTER(abi.Dims), C.POINTER(abi.Params), C.POINTER(abi.Grids), DP, DP,
            C.POINTER(C.c_int32), C.c_double, C.POINTER(abi.EpStats), C.c_int, C.c_char_p]
        lib.orc_update_energetic_particles_news.restype = C.c_int
        lib.orc_update_mhd.argtypes = [C.POINTER(abi.Dims), C.POINTER(abi.Params), DP, C.c_double]
        lib.orc_update_mhd_curl.argtypes = [C.POINTER(abi.Dims), C.POINTER(abi.Params), DP,
                                            C.c_double, DP]
        lib.orc_update_energetic_particles_perp.argtypes = [
            C.POINTER(abi.Dims), C.POINTER(abi.Params), C.POINTER(abi.Grids), DP, DP,
            C.POINTER(C.c_int32), C.c_int, C.c_double, C.POINTER(abi.DriftParams), DP,
            C.POINTER(abi.EpStats), C.c_int, C.c_char_p]
        lib.orc_update_energetic_particles_perp.restype = C.c_int
        lib.orc_move_nodes.argtypes = [C.POINTER(abi.Dims), C.POINTER(abi.Params), DP, C.c_double]
        lib.orc_omni_flux.argtypes = [C.POINTER(abi.Dims), C.POINTER(abi.Grids), DP, DP]
        lib.orc_omni_flux.restype = None
        lib.orc_seed_function.argtypes = [C.POINTER(abi.Params), C.c_double, C.c_double]
        lib.orc_seed_function.restype = C.c_double
        lib.orc_build_grids.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                        C.c_double, C.c_double, DP, DP, DP, DP, DP, DP, DP, DP]
        lib.orc_build_grids.restype = None
        _mas_bind(lib)
        self.lib = lib

    def mas_update_mhd(self, dims, params, nodes, mas: MasState, t_global=0.0):
        return self.lib.orc_mas_update_mhd(C.byref(dims), C.byref(params), _dp(nodes),
                                           C.byref(mas), t_global)

    def mas_move_nodes(self, dims, params, nodes, mas: MasState, dt):
        return self.lib.orc_mas_move_nodes(C.byref(dims), C.byref(params), _dp(nodes),
                                           C.byref(mas), dt)

    def grids(self, E, M, e_min, e_max, mass=1.0, charge=1.0, rigidity_power=1.0 / 3.0):
        out = {k: np.zeros(E) for k in ("egrid", "vgrid", "vgrid_i", "pgrid", "rigidity")}
        out["mugrid"] = np.zeros(M)
        dl, dm = C.c_double(), C.c_double()
        self.lib.orc_build_grids(E, M, e_min, e_max, mass, charge, rigidity_power,
                                 _dp(out["egrid"]), _dp(out["vgrid"]), _dp(out["vgrid_i"]),
                                 _dp(out["pgrid"]), _dp(out["rigidity"]), _dp(out["mugrid"]),
                                 C.byref(dl), C.byref(dm))
        out["dlnp"], out["dmu"] = dl.value, dm.value
        return out

    def update_energetic_particles(self, dims, params, grids_s, f, nodes, nthreads=1,
                                   streams=None, news=None, kperxkpar=0.01):
        """news: S x 4 NEWS neighbour stream indices to diffuse across shells
        (DiffuseShellData) after every sub-step; None leaves it off."""
        st = abi.EpStats()
        st.min_tau = np.finfo(np.float64).max
        err = C.create_string_buffer(256)
        if news is not None:
            nw = np.ascontiguousarray(news, dtype=np.int32)
            assert streams is None and nw.shape == (dims.num_streams, 4)
            rc = self.lib.orc_update_energetic_particles_news(
                C.byref(dims), C.byref(params), C.byref(grids_s), _dp(f), _dp(nodes),
                nw.ctypes.data_as(C.POINTER(C.c_int32)), kperxkpar, C.byref(st), nthreads, err)
            return rc, st, err.value.decode()
        s0, s1 = (0, dims.num_streams) if streams is None else streams
        rc = self.lib.orc_update_energetic_particles_range(
            C.byref(dims), C.byref(params), C.byref(grids_s), _dp(f), _dp(nodes), s0, s1,
            C.byref(st), nthreads, err)
        return rc, st, err.value.decode()

    def update_mhd(self, dims, params, nodes, t_global, curl=None):
        """curl: a (3, S*N) array to receive curl(B)/B^2 (useDrift), or None."""
        if curl is not None:
            return self.lib.orc_update_mhd_curl(C.byref(dims), C.byref(params), _dp(nodes),
                                                t_global, _dp(curl))
        return self.lib.orc_update_mhd(C.byref(dims), C.byref(params), _dp(nodes), t_global)

    def update_energetic_particles_perp(self, dims, params, grids_s, f, nodes, news,
                                        kperxkpar=None, drift=None, curl=None, nthreads=1):
        """The update with the perpendicular steps: shell diffusion when
        kperxkpar is given, drift when drift (abi.DriftParams) and curl are."""
        st = abi.EpStats()
        st.min_tau = np.finfo(np.float64).max
        err = C.create_string_buffer(256)
        nw = np.ascontiguousarray(news, dtype=np.int32)
        rc = self.lib.orc_update_energetic_particles_perp(
            C.byref(dims), C.byref(params), C.byref(grids_s), _dp(f), _dp(nodes),
            nw.ctypes.data_as(C.POINTER(C.c_int32)), int(kperxkpar is not None),
            float(kperxkpar or 0.0), C.byref(drift) if drift is not None else None,
            _dp(curl) if curl is not None else None, C.byref(st), nthreads, err)
        return rc, st, err.value.decode()

    def move_nodes(self, dims, params, nodes, dt):
        return self.lib.orc_move_nodes(C.byref(dims), C.byref(params), _dp(nodes), dt)

    def omni_flux(self, dims, grids_s, f):
        out = np.zeros(dims.num_streams * dims.num_nodes * dims.num_energies)
        self.lib.orc_omni_flux(C.byref(dims), C.byref(grids_s), _dp(f), _dp(out))
        return out

    def seed_function(self, params, energy, r):
        return self.lib.orc_seed_function(C.byref(params), energy, r)


class MasState(C.Structure):
    """orc_mas_t of eprem_oracle.h."""
    _fields_ = [("slot0", C.POINTER(abi.MasSlice)), ("slot1", C.POINTER(abi.MasSlice)),
                ("s_cor", C.c_double), ("phi_offset", C.c_double), ("p", abi.MasParams)]


def _mas_bind(lib):
    lib.orc_mas_update_mhd.argtypes = [C.POINTER(abi.Dims), C.POINTER(abi.Params), DP,
                                       C.POINTER(MasState), C.c_double]
    lib.orc_mas_move_nodes.argtypes = [C.POINTER(abi.Dims), C.POINTER(abi.Params), DP,
                                       C.POINTER(MasState), C.c_double]


class Reference:
    """The reference's own updateEnergeticParticles / updateMhd / moveNodes.
    The reference allocates its globals once per process, so one process can
    host one configuration; tests run it in a child process."""

    def __init__(self, path: str = REF_LIB):
        lib = C.CDLL(path)
        lib.ref_setup.argtypes = [C.c_int, C.c_int, C.POINTER(abi.Dims), C.POINTER(abi.Params),
                                  C.c_double, C.c_double, C.c_double, C.c_double, C.c_double]
        lib.ref_get_grids.argtypes = [DP] * 5 + [DP, DP]
        lib.ref_load.argtypes = [DP, DP]
        lib.ref_store.argtypes = [DP, DP]
        lib.ref_update_energetic_particles.argtypes = [C.c_double, C.POINTER(abi.EpStats)]
        lib.ref_update_mhd.argtypes = [C.c_double]
        lib.ref_move_nodes.argtypes = [C.c_double]
        lib.ref_mas_setup.argtypes = [C.POINTER(abi.MasParams), C.POINTER(abi.MasSlice),
                                      C.POINTER(abi.MasSlice), C.c_double, C.c_double]
        lib.ref_mas_move_nodes.argtypes = [C.c_double]
        lib.ref_shell_diffusion.argtypes = [C.c_int, C.c_double, C.POINTER(C.c_int32)]
        lib.ref_drift.argtypes = [C.c_int, C.POINTER(C.c_int32), C.POINTER(C.c_double)]
        self.lib = lib

    def drift(self, num_streams):
        """Switch DriftShellData on; returns the reference's NEWS links and
        its lnpmin."""
        news = np.zeros((num_streams, 4), dtype=np.int32)
        lnpmin = C.c_double()
        self.lib.ref_drift(1, news.ctypes.data_as(C.POINTER(C.c_int32)), C.byref(lnpmin))
        return news, lnpmin.value

    def shell_diffusion(self, kperxkpar, num_streams):
        """Switch on DiffuseShellData; returns the reference's NEWS links
        (num_streams x 4 stream indices: north, east, west, south)."""
        news = np.zeros((num_streams, 4), dtype=np.int32)
        self.lib.ref_shell_diffusion(1, kperxkpar, news.ctypes.data_as(C.POINTER(C.c_int32)))
        return news

    def mas_setup(self, mp, s0, s1, s_cor, phi_offset):
        self._mas_keep = (mp, s0, s1)
        return self.lib.ref_mas_setup(C.byref(mp), C.byref(s0), C.byref(s1), s_cor, phi_offset)

    def mas_move_nodes(self, dt):
        self.lib.ref_mas_move_nodes(dt)

    def setup(self, w, precision=abi.EPREM_FP64):
        d = w.dims(precision)
        rc = self.lib.ref_setup(w.rows, w.cols, C.byref(d), C.byref(w.params), w.e_min, w.e_max,
                                w.mass, w.charge, w.rigidity_power)
        if rc:
            raise RuntimeError(f"ref_setup failed: {rc}")
        E, M = w.num_energies, w.num_mu
        g = {k: np.zeros(E) for k in ("egrid", "vgrid", "vgrid_i", "rigidity")}
        g["mugrid"] = np.zeros(M)
        dl, dm = C.c_double(), C.c_double()
        self.lib.ref_get_grids(_dp(g["egrid"]), _dp(g["vgrid"]), _dp(g["vgrid_i"]),
                               _dp(g["mugrid"]), _dp(g["rigidity"]), C.byref(dl), C.byref(dm))
        g["dlnp"], g["dmu"] = dl.value, dm.value
        return g

    def load(self, f, nodes):
        self.lib.ref_load(_dp(f), _dp(nodes))

    def store(self, f, nodes):
        self.lib.ref_store(_dp(f), _dp(nodes))

    def update_energetic_particles(self, t_global=0.0):
        st = abi.EpStats()
        rc = self.lib.ref_update_energetic_particles(t_global, C.byref(st))
        return rc, st

    def update_mhd(self, t_global):
        self.lib.ref_update_mhd(t_global)

    def move_nodes(self, dt):
        self.lib.ref_move_nodes(dt)
