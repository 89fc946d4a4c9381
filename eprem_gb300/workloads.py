"""Synthetic run states for the energetic-particle update.

There is no public dataset behind this path: the reference's inputs are a
config file plus an analytic (Parker) or MAS background, and its regression
cases are end-to-end runs.  These generators build the same kind of state
directly -- node positions along Parker spirals rooted at the cube-sphere
stream footpoints, the analytic MHD fields on those nodes, and a seed-function
distribution with a seeded 1% perturbation -- with the sizes of the workloads
this project measures:

* ``small``  -- 24 streams x 400 nodes, 20 energies (0.1-100 MeV) x 20 mu
  (the CPU-runnable plain-method case);
* ``scale``  -- 1536 streams x 1000 nodes, 50 energies (0.1-1000 MeV) x 40 mu
  (the precision-at-scale case the headline number is measured on);
* ``testsuite-like`` variants with the wind / cone parameters of the
  reference's regression inputs (testsuite/*/input/eprem_input_file).

Units follow the reference (src/baseTypes.h): positions in rScale units,
times in AU/c, speeds in c, B in MHD_B_NORM, density in cm^-3.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

from . import abi

# src/baseTypes.h:47-115
PI = 3.1415926535897932
MP = 1.6726e-24
MEV = 1.6022e-6
GEV = 1.6022e-3
C_LIGHT = 2.99792458e10
AU = 1.495978707e13
TAU = AU / C_LIGHT
DAY = TAU / (24.0 * 60.0 * 60.0)
MZERO = MP * C_LIGHT * C_LIGHT / GEV
MHD_DENSITY_NORM = 1.0
MHD_B_NORM = math.sqrt(MP * MHD_DENSITY_NORM) * C_LIGHT
MAS_TIME_NORM = 1445.87003080685
OMEGA_SUN_DEFAULT = (0.004144 / MAS_TIME_NORM) * TAU


def splitmix64(seed: int, n: int) -> np.ndarray:
    """n outputs of the splitmix64 generator started at `seed` (uint64)."""
    with np.errstate(over="ignore"):
        idx = np.arange(1, n + 1, dtype=np.uint64)
        z = np.uint64(seed) + idx * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return z


def uniform_pm1(seed: int, n: int) -> np.ndarray:
    """U(-1, 1) doubles from the top 53 bits of splitmix64."""
    u = (splitmix64(seed, n) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
    return 2.0 * u - 1.0


@dataclasses.dataclass
class Workload:
    name: str
    rows: int
    cols: int
    num_nodes: int
    num_energies: int
    num_mu: int
    e_min: float
    e_max: float
    r_min_au: float
    r_max_au: float
    params: abi.Params
    mass: float = 1.0
    charge: float = 1.0
    rigidity_power: float = 1.0 / 3.0
    seed: int = 12345
    perturb: float = 0.01
    cluster_inner: int = 0  # nodes packed near r_min (exercises thinning)

    @property
    def num_streams(self) -> int:
        return 6 * self.rows * self.cols

    def dims(self, precision: int = abi.EPREM_FP64) -> abi.Dims:
        return abi.Dims(self.num_streams, self.num_nodes, 1, self.num_energies, self.num_mu,
                        precision)

    @property
    def cells(self) -> int:
        return self.num_streams * self.num_nodes * self.num_energies * self.num_mu


def default_params() -> abi.Params:
    """getParams defaults (src/configuration.c:58-217) after
    setRuntimeConstants (:325-348)."""
    p = abi.Params()
    p.r_scale = 0.005
    p.t_del = 0.01041666666667 / DAY
    p.num_ep_steps = 30
    p.use_parallel_diffusion = 1
    p.use_adiabatic_focus = 1
    p.use_adiabatic_change = 1
    p.check_seed_population = 1
    p.use_ep_boundary = 1
    p.use_boundary_function = 1
    p.adiabatic_focus_alg = 1
    p.adiabatic_change_alg = 1
    p.damp_cooling = 0.0
    p.dsh_min = 5.0e-5
    p.mfp_type = 1
    p.lamo = 1.0
    p.mfp_radial_power = 2.0
    p.mfp_b_power = 0.75
    p.mhd_bs_au = 1.60e-5 / MHD_B_NORM
    p.bf_amplitude = 1.0
    p.bf_xi = 1.0
    p.bf_gamma = 2.0
    p.bf_beta = 1.7
    p.bf_ecutoff = 1.0
    p.bf_r0 = 1.0
    p.mhd_us = 400.0e5 / C_LIGHT
    p.mhd_ns_au = 8.30 / MHD_DENSITY_NORM
    p.omega_sun = OMEGA_SUN_DEFAULT
    p.ideal_shock = 0
    p.ideal_shock_sharpness = 1.0
    p.ideal_shock_scale_length = 0.0046491
    p.ideal_shock_jump = 4.0
    p.ideal_shock_falloff = 0.0
    p.ideal_shock_speed = 1500e5
    p.ideal_shock_init_time = 0.0
    p.ideal_shock_theta = 1.570796
    p.ideal_shock_phi = 0.0
    p.ideal_shock_width = 0.0
    p.max_subcycles = 0
    return p


def _plain_wind_params(flow_kms=400.0, b_equator_nt=5.0, density=5.0) -> abi.Params:
    """Analytic wind of the plain-method workloads: 400 km/s, |B| = 5 nT at
    1 AU in the equator (Br chosen through the Parker angle), n = 5 cm^-3 at
    1 AU; lambda_par = 0.3 AU at 1 GV scaling as R^(1/3) with no r scaling
    (mfpRadialPower at 1e-30, above its configuration minimum of 1e-33); seed
    a pure power law of index -3.5 (cutoff at 1e9 MeV)."""
    p = default_params()
    p.mhd_us = flow_kms * 1e5 / C_LIGHT
    omega_r_over_v = p.omega_sun * 1.0 / p.mhd_us
    br_gauss = b_equator_nt * 1e-5 / math.sqrt(1.0 + omega_r_over_v ** 2)
    p.mhd_bs_au = br_gauss / MHD_B_NORM
    p.mhd_ns_au = density / MHD_DENSITY_NORM
    p.lamo = 0.3
    p.mfp_type = 1
    p.mfp_radial_power = 1e-30
    p.bf_gamma = 3.5
    p.bf_ecutoff = 1e9
    p.bf_xi = 1.0
    p.bf_beta = 1.7
    return p


def small_plain() -> Workload:
    """24 streams x 400 nodes x 20 E x 20 mu, 0.05-5 AU, 24 h of 96 steps."""
    return Workload("plain-small 24x400x20x20", 2, 2, 400, 20, 20, 0.1, 100.0, 0.05, 5.0,
                    _plain_wind_params())


def scale_plain() -> Workload:
    """1536 streams x 1000 nodes x 50 E (0.1-1000 MeV) x 40 mu."""
    return Workload("precision-at-scale 1536x1000x50x40", 16, 16, 1000, 50, 40, 0.1, 1000.0,
                    0.05, 5.0, _plain_wind_params())


def custom(rows, cols, nodes, energies, mu, e_min=0.1, e_max=100.0, r_min=0.05, r_max=5.0,
           name=None, **param_overrides) -> Workload:
    p = _plain_wind_params()
    for k, v in param_overrides.items():
        setattr(p, k, v)
    return Workload(name or f"custom {6*rows*cols}x{nodes}x{energies}x{mu}", rows, cols, nodes,
                    energies, mu, e_min, e_max, r_min, r_max, p)


def testsuite_like(case: str, rows=2, cols=2, nodes=60) -> Workload:
    """Parameters of the reference regression inputs
    (testsuite/{wind,cone}/input/eprem_input_file), on synthetic geometry."""
    p = default_params()
    p.r_scale = 0.00465047
    p.mhd_bs_au = 1.60e-5 / MHD_B_NORM
    p.mhd_ns_au = 8.30
    p.lamo = 1.0
    p.bf_amplitude = 1.0
    p.bf_xi = 0.10
    p.bf_gamma = 2.0
    p.bf_beta = 1.7
    p.bf_ecutoff = 1.0
    p.omega_sun = 0.001429813
    if case == "wind":
        p.mhd_us = 500.0e5 / C_LIGHT
        p.t_del = 0.041666666666667 / DAY
        p.num_ep_steps = 5
        return Workload("wind-like", rows, cols, nodes, 12, 6, 1.0, 200.0, 0.01, 1.0, p,
                        cluster_inner=6)
    if case == "cone":
        p.mhd_us = 300.0e5 / C_LIGHT
        p.t_del = 0.010416666666667 / DAY
        p.num_ep_steps = 20
        p.ideal_shock = 1
        p.ideal_shock_sharpness = 1.0
        p.ideal_shock_scale_length = 0.0046491
        p.ideal_shock_jump = 2.9
        p.ideal_shock_speed = 0.9e8
        p.ideal_shock_init_time = 0.5
        return Workload("cone-like", 1, 1, nodes, 12, 8, 1.0, 200.0, 0.01, 1.2, p,
                        cluster_inner=4)
    raise ValueError(case)


# ---------------------------------------------------------------------------
def build_grids(w: Workload):
    """initEnergeticParticlesGrids (src/energeticParticlesInit.c:36-100).
    Returns a dict of numpy arrays plus dlnp, dmu."""
    E, M = w.num_energies, w.num_mu
    kin = w.e_min * MEV / (MP * C_LIGHT * C_LIGHT)
    lnpmin = math.log(math.sqrt(kin * kin + 2.0 * kin))
    kin = w.e_max * MEV / (MP * C_LIGHT * C_LIGHT)
    lnpmax = math.log(math.sqrt(kin * kin + 2.0 * kin))
    dlnp = (lnpmax - lnpmin) / (E - 1.0)
    egrid = np.empty(E); vgrid = np.empty(E); vgrid_i = np.empty(E); rig = np.empty(E)
    for e in range(E):
        p = math.exp(lnpmin + e * dlnp)
        egrid[e] = math.sqrt(1.0 + p * p) - 1.0
        vgrid[e] = p / math.sqrt(1.0 + p * p)
        vgrid_i[e] = math.sqrt(1.0 + p * p) / p
        r = (w.mass / w.charge) * p * MZERO
        rig[e] = r ** w.rigidity_power
    dmu = 2.0 / (1.0 * M)
    mugrid = np.array([0.5 * ((-1.0 + (m + 1.0) * dmu) + (-1.0 + m * dmu)) for m in range(M)])
    return {"egrid": egrid, "vgrid": vgrid, "vgrid_i": vgrid_i, "mugrid": mugrid,
            "rigidity": rig, "dlnp": dlnp, "dmu": dmu, "lnpmin": lnpmin}


def drift_params(w: Workload, g: dict) -> abi.DriftParams:
    """eprem_drift_params_t of the workload (useDrift): lnpmin of its momentum
    grid and the species' charge and mass."""
    return abi.DriftParams(g["lnpmin"], w.charge, w.mass)


def grids_struct(g) -> tuple[abi.Grids, list]:
    """ctypes Grids pointing at the numpy arrays of `g` (keep the list alive)."""
    keep = []
    def ptr(name):
        a = np.ascontiguousarray(g[name], dtype=np.float64)
        keep.append(a)
        return a.ctypes.data_as(abi.C.POINTER(abi.C.c_double))
    s = abi.Grids(ptr("egrid"), ptr("vgrid"), ptr("vgrid_i"), ptr("mugrid"), ptr("rigidity"),
                  float(g["dlnp"]), float(g["dmu"]))
    return s, keep


def stream_footpoints(rows: int, cols: int):
    """(theta, phi) of the cube-sphere cell centres, computeLines order
    (face-major, then row, then col; src/unifiedOutput.c:64-92)."""
    out = []
    for face in range(6):
        for row in range(rows):
            for col in range(cols):
                u = -1.0 + (2.0 * col + 1.0) / cols
                v = -1.0 + (2.0 * row + 1.0) / rows
                if face == 0: x, y, z = 1.0, u, v
                elif face == 1: x, y, z = -u, 1.0, v
                elif face == 2: x, y, z = -1.0, -u, v
                elif face == 3: x, y, z = u, -1.0, v
                elif face == 4: x, y, z = -v, u, 1.0
                else: x, y, z = v, u, -1.0
                n = math.sqrt(x * x + y * y + z * z)
                out.append((math.acos(z / n), math.atan2(y, x) % (2 * PI)))
    return out


def node_radii(w: Workload) -> np.ndarray:
    """Log-uniform radii from r_min to r_max (AU); with cluster_inner > 0 the
    first nodes sit far closer together than dsh_min, as the reference's
    node seeding leaves them near the inner boundary."""
    N = w.num_nodes
    r = w.r_min_au * (w.r_max_au / w.r_min_au) ** (np.arange(N) / (N - 1.0))
    if w.cluster_inner:
        k = np.arange(w.cluster_inner)
        r[: w.cluster_inner] = w.r_min_au * (1.0 + 1e-6 * k)
        r[w.cluster_inner:] = np.maximum(r[w.cluster_inner:], w.r_min_au * 1.001)
    return r


def initial_nodes(w: Workload) -> np.ndarray:
    """[NODE_NFIELDS, S*N] with positions along Parker spirals; MHD fields
    zero (fill them with update_mhd before use)."""
    S, N = w.num_streams, w.num_nodes
    p = w.params
    nodes = np.zeros((abi.NODE_NFIELDS, S * N))
    r = node_radii(w)
    for s, (th, ph0) in enumerate(stream_footpoints(w.rows, w.cols)):
        ph = ph0 - p.omega_sun * r / p.mhd_us
        x = r * math.sin(th) * np.cos(ph) / p.r_scale
        y = r * math.sin(th) * np.sin(ph) / p.r_scale
        z = r * math.cos(th) * np.ones_like(r) / p.r_scale
        sl = slice(s * N, (s + 1) * N)
        nodes[abi.NODE["RX"], sl] = x
        nodes[abi.NODE["RY"], sl] = y
        nodes[abi.NODE["RZ"], sl] = z
        nodes[abi.NODE["RMAG"], sl] = np.sqrt(x * x + y * y + z * z)
    return nodes


def seed_function(p: abi.Params, energy, r):
    """sepSeedFunction (src/energeticParticlesBoundary.c:67-116), vectorised;
    used to build initial distributions, not as a checker."""
    efac = MEV / (MP * C_LIGHT * C_LIGHT)
    normJ0 = p.bf_amplitude * (MP * C_LIGHT) / (MHD_DENSITY_NORM * MEV)
    normRadius = p.bf_r0 / p.r_scale
    radial = np.power(r / normRadius, -p.bf_beta)
    power = np.power(energy / (1.0 * efac), -p.bf_gamma)
    expt = np.exp(-(energy / (p.bf_ecutoff * efac)))
    f = normJ0 * radial * power * expt / p.bf_xi / (2.0 * energy)
    return np.maximum(f, np.finfo(np.float64).tiny)


def initial_f(w: Workload, nodes: np.ndarray, grids) -> np.ndarray:
    """Seed function at each (stream, node, E), isotropic in mu, times
    (1 + perturb * U(-1,1)) drawn per (stream, node, E) from splitmix64."""
    S, N, E, M = w.num_streams, w.num_nodes, w.num_energies, w.num_mu
    rmag = nodes[abi.NODE["RMAG"]].reshape(S, N)
    f = seed_function(w.params, grids["egrid"][None, None, :], rmag[:, :, None])
    f = f * (1.0 + w.perturb * uniform_pm1(w.seed, S * N * E).reshape(S, N, E))
    return np.ascontiguousarray(np.broadcast_to(f[..., None], (S, N, E, M))).reshape(-1)


def fill_initial_f(w: Workload, nodes: np.ndarray, grids, out: np.ndarray,
                   streams_per_chunk: int = 64) -> np.ndarray:
    """initial_f written into `out` (length S*N*E*M) stream chunk by stream
    chunk, so that large workloads need no full-size temporaries."""
    S, N, E, M = w.num_streams, w.num_nodes, w.num_energies, w.num_mu
    rmag = nodes[abi.NODE["RMAG"]].reshape(S, N)
    pert = uniform_pm1(w.seed, S * N * E).reshape(S, N, E)
    view = out.reshape(S, N, E, M)
    for s0 in range(0, S, streams_per_chunk):
        s1 = min(S, s0 + streams_per_chunk)
        f = seed_function(w.params, grids["egrid"][None, None, :], rmag[s0:s1, :, None])
        view[s0:s1] = (f * (1.0 + w.perturb * pert[s0:s1]))[..., None]
    return out



def with_faces(w: Workload, rows: int, cols: int) -> Workload:
    """The same per-stream workload on a 6 x rows x cols cube-sphere (fewer or
    more streams, each with identical node, energy and mu grids)."""
    return dataclasses.replace(w, rows=rows, cols=cols,
                               name=f"{w.name} on {6 * rows * cols} streams")


# ---------------------------------------------------------------------------
# Synthetic MAS-like background (the MHD-coupled workload).  MAS output is a
# set of HDF5 slices per field on staggered spherical meshes in MAS units
# (src/readMAS.c, src/baseTypes.h:104-115).  This builds the same structure
# from an analytic Parker wind plus a Gaussian-shell CME pulse: the CME doubles
# the density and adds a radial speed increment inside a shell launched at
# 2 Rs that moves outward at the CME speed, within a cone of given half-width.
MAS_LENGTH_NORM = 6.96e10
MAS_RHO_NORM = 1.6726e-16
RSUN = 6.96e10
RSAU = RSUN / AU
MAS_B_CONVERT = math.sqrt(4.0 * PI * MAS_RHO_NORM) * MAS_LENGTH_NORM / MAS_TIME_NORM / MHD_B_NORM
MAS_V_CONVERT = (MAS_LENGTH_NORM / MAS_TIME_NORM) / C_LIGHT
MAS_RHO_CONVERT = (MAS_RHO_NORM / MP) / MHD_DENSITY_NORM


@dataclasses.dataclass
class MasGrid:
    nr: int
    nt: int
    np_: int
    r_min_rs: float
    r_max_rs: float
    times: np.ndarray               # slice times (AU/c)
    params: "abi.MasParams"
    wind: abi.Params
    cme_speed_kms: float = 1500.0
    cme_dv_kms: float = 1200.0
    cme_density_factor: float = 2.0
    cme_half_width_deg: float = 30.0
    cme_launch_rs: float = 2.0
    cme_theta: float = PI / 2
    cme_phi: float = 0.0

    def meshes(self):
        """Cell-centre meshes and the half-shifted ones of the staggered
        components: r (solar radii, geometric stretch), theta, phi."""
        rf = self.r_min_rs * (self.r_max_rs / self.r_min_rs) ** (np.arange(self.nr) / (self.nr - 1))
        rh = np.sqrt(rf * np.concatenate([rf[1:], [rf[-1] * rf[-1] / rf[-2]]]))
        dt_ = PI / self.nt
        tc = (np.arange(self.nt) + 0.5) * dt_
        th = np.arange(self.nt) * dt_ + dt_  # half-shifted
        th[-1] = min(th[-1], PI)
        dp = 2 * PI / self.np_
        pc = (np.arange(self.np_) + 0.5) * dp
        ph = np.arange(self.np_) * dp + dp
        return {"r": rf, "rh": rh, "t": tc, "th": th, "p": pc, "ph": ph}

    def field_meshes(self):
        m = self.meshes()
        # staggered by half a cell along each vector component's own direction
        return {"Bp": (m["r"], m["t"], m["ph"]), "Bt": (m["r"], m["th"], m["p"]),
                "Br": (m["rh"], m["t"], m["p"]), "Vp": (m["r"], m["t"], m["ph"]),
                "Vt": (m["r"], m["th"], m["p"]), "Vr": (m["rh"], m["t"], m["p"]),
                "rho": (m["r"], m["t"], m["p"])}

    def slice_fields(self, t: float) -> dict:
        """All seven fields at time t (AU/c), MAS units, float32 [phi][theta][r]."""
        w = self.wind
        out = {}
        shell_r = self.cme_launch_rs + self.cme_speed_kms * 1e5 * (t * TAU) / RSUN
        ct0, st0 = math.cos(self.cme_theta), math.sin(self.cme_theta)
        shape = (len(self.field_meshes()["rho"][2]), len(self.field_meshes()["rho"][1]),
                 len(self.field_meshes()["rho"][0]))
        for name, (mr, mt, mp) in self.field_meshes().items():
            # broadcast views [phi][theta][r] (the values a full meshgrid holds)
            P, Tt, R = mp[:, None, None], mt[None, :, None], mr[None, None, :]
            r_au = R * RSAU
            cos_ang = np.cos(Tt) * ct0 + np.sin(Tt) * st0 * np.cos(P - self.cme_phi)
            ang = np.arccos(np.clip(cos_ang, -1.0, 1.0))
            hw = math.radians(self.cme_half_width_deg)
            g = np.exp(-((R - shell_r) / 1.0) ** 2) * np.exp(-(ang / hw) ** 2)
            vr = w.mhd_us * (1.0 + 0.0 * R) + self.cme_dv_kms * 1e5 / C_LIGHT * g
            br = w.mhd_bs_au / (r_au * r_au)
            if name == "Br":
                val = br / MAS_B_CONVERT
            elif name == "Bt":  # weak latitudinal field so every component is exercised
                val = (0.05 * br * np.sin(P)) / MAS_B_CONVERT
            elif name == "Bp":
                val = (-1.0 * r_au * br * (w.omega_sun / vr) * np.sin(Tt)) / MAS_B_CONVERT
            elif name == "Vr":
                val = vr / MAS_V_CONVERT
            elif name == "Vt":
                val = (5.0e5 / C_LIGHT) * np.sin(P) / MAS_V_CONVERT
            elif name == "Vp":
                val = (10.0e5 / C_LIGHT) * np.cos(Tt) / MAS_V_CONVERT
            else:
                val = (w.mhd_ns_au / (r_au * r_au)) * (1.0 + (self.cme_density_factor - 1.0) * g)
                val = val / MAS_RHO_CONVERT
            out[name] = np.ascontiguousarray(np.broadcast_to(val, shape), dtype=np.float32)
        return out


def mas_grid(nr=300, nt=180, np_=360, r_min_rs=1.0, r_max_rs=30.0, n_slices=16,
             slice_dt_hours=1.0, wind: abi.Params | None = None, **kw) -> MasGrid:
    p = abi.MasParams()
    p.radial_max = r_max_rs
    p.v_min = 50.0e5
    p.cor_rotate_fake = 0
    p.rotate_solution = 1
    p.max_slices = n_slices
    times = np.arange(n_slices) * slice_dt_hours * 3600.0 / TAU
    return MasGrid(nr, nt, np_, r_min_rs, r_max_rs, times, p, wind or _plain_wind_params(), **kw)


def mas_slice_struct(grid: MasGrid, fields: dict):
    """abi.MasSlice over `fields` (keep the returned list alive)."""
    keep = []
    s = abi.MasSlice()
    fm = grid.field_meshes()
    for i, name in enumerate(abi.MAS_FIELDS):
        meshes = [np.ascontiguousarray(m, dtype=np.float32) for m in fm[name]]
        data = fields[name]
        keep.extend(meshes)
        keep.append(data)
        for ax in range(3):
            s.dims[i][ax] = len(meshes[ax])
            s.mesh[i][ax] = meshes[ax].ctypes.data_as(abi.C.POINTER(abi.C.c_float))
        s.data[i] = data.ctypes.data_as(abi.C.POINTER(abi.C.c_float))
    return s, keep


def mas_workload(streams_rows=2, streams_cols=2, nodes=60, energies=12, mu=8, r_min_au=0.006,
                 r_max_au=1.0, name=None) -> Workload:
    """Nodes from inside the MAS domain out past its edge (masWind takes over
    beyond masRadialMax)."""
    p = _plain_wind_params()
    return Workload(name or f"mas {6 * streams_rows * streams_cols}x{nodes}x{energies}x{mu}",
                    streams_rows, streams_cols, nodes, energies, mu, 0.1, 100.0, r_min_au,
                    r_max_au, p)


def ensemble_members(n: int = 64, seed: int = 20240607) -> list[Workload]:
    """The batched-ensemble workload: n independent runs with uneven sizes and
    parameters drawn from splitmix64(seed) -- streams 6 r^2 with r log-uniform
    in [2, 16] (24-1536 streams), 400-2000 nodes, 20-50 energies, 20-40 mu
    cells, seed-spectrum index -[2.5, 4], lambda_parallel 0.05-1 AU at 1 GV,
    and an ideal shock (a CME-driven front in the analytic wind, 30-degree
    half-width) at 800-2500 km/s."""
    u = 0.5 * (uniform_pm1(seed, 8 * n).reshape(n, 8) + 1.0)  # U(0, 1)
    out = []
    for i in range(n):
        r = int(round(2.0 * 8.0 ** u[i, 0]))
        nodes = 400 + int(u[i, 1] * 1600.999)
        E = 20 + int(u[i, 2] * 30.999)
        M = 20 + int(u[i, 3] * 20.999)
        p = _plain_wind_params()
        p.bf_gamma = 2.5 + 1.5 * u[i, 4]
        p.lamo = 0.05 + 0.95 * u[i, 5]
        p.ideal_shock = 1
        p.ideal_shock_speed = (800.0 + 1700.0 * u[i, 6]) * 1e5
        p.ideal_shock_jump = 2.9
        p.ideal_shock_init_time = 0.0
        p.ideal_shock_theta = PI / 2
        p.ideal_shock_phi = 2.0 * PI * u[i, 7]
        p.ideal_shock_width = 2.0 * math.radians(30.0)
        w = Workload(f"member {i}: {6 * r * r}x{nodes}x{E}x{M}", r, r, nodes, E, M, 0.1,
                     1000.0, 0.05, 5.0, p, seed=seed + i)
        out.append(w)
    return out


def ensemble_members_small(n: int = 64, seed: int = 20240611) -> list[Workload]:
    """A parameter sweep of n runs of the CPU-runnable case's size (24 streams
    x 400 nodes x 20 E x 20 mu, 0.1-100 MeV, 0.05-5 AU): seed-spectrum index
    -[2.5, 4], lambda_parallel 0.05-1 AU at 1 GV and an ideal shock at
    800-2500 km/s drawn from splitmix64(seed).  Each run alone holds 480
    (stream, energy) slabs, about three per SM: too few to fill the GPU,
    which is where one launch over all runs' slabs pays."""
    u = 0.5 * (uniform_pm1(seed, 4 * n).reshape(n, 4) + 1.0)
    out = []
    for i in range(n):
        p = _plain_wind_params()
        p.bf_gamma = 2.5 + 1.5 * u[i, 0]
        p.lamo = 0.05 + 0.95 * u[i, 1]
        p.ideal_shock = 1
        p.ideal_shock_speed = (800.0 + 1700.0 * u[i, 2]) * 1e5
        p.ideal_shock_jump = 2.9
        p.ideal_shock_init_time = 0.0
        p.ideal_shock_theta = PI / 2
        p.ideal_shock_phi = 2.0 * PI * u[i, 3]
        p.ideal_shock_width = 2.0 * math.radians(30.0)
        out.append(Workload(f"small member {i}: 24x400x20x20", 2, 2, 400, 20, 20, 0.1, 100.0,
                            0.05, 5.0, p, seed=seed + i))
    return out
