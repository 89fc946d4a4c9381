"""ctypes mirror of include/eprem_gpu.h.

The structs and constants here must match the C header field for field; the
CPU test suite checks the sizes against the compiled library.
"""
import ctypes as C

EPREM_GPU_OK = 0
EPREM_GPU_ERR_ARG = -1
EPREM_GPU_ERR_CUDA = -2
EPREM_GPU_ERR_NAN = -3
EPREM_GPU_ERR_INF = -4
EPREM_GPU_ERR_DS = -5
EPREM_GPU_ERR_SUBCYCLES = -6
EPREM_GPU_ERR_UNSUPPORTED = -7
EPREM_GPU_ERR_STATE = -8

STATUS_NAMES = {
    EPREM_GPU_OK: "ok",
    EPREM_GPU_ERR_ARG: "bad argument",
    EPREM_GPU_ERR_CUDA: "CUDA failure",
    EPREM_GPU_ERR_NAN: "NaN in distribution",
    EPREM_GPU_ERR_INF: "Inf in distribution",
    EPREM_GPU_ERR_DS: "ds underflow",
    EPREM_GPU_ERR_SUBCYCLES: "sub-cycle cap exceeded",
    EPREM_GPU_ERR_UNSUPPORTED: "unsupported option",
    EPREM_GPU_ERR_STATE: "stream thinned below 3 nodes",
}

EPREM_FP64 = 0
EPREM_FP32 = 1
FLUX_STATIC_MAX = 1048576  # EPREM_GPU_FLUX_STATIC_MAX


class Dims(C.Structure):
    _fields_ = [
        ("num_streams", C.c_int32),
        ("num_nodes", C.c_int32),
        ("num_species", C.c_int32),
        ("num_energies", C.c_int32),
        ("num_mu", C.c_int32),
        ("precision", C.c_int32),
    ]


class Params(C.Structure):
    _fields_ = [
        ("r_scale", C.c_double),
        ("t_del", C.c_double),
        ("num_ep_steps", C.c_int32),
        ("use_parallel_diffusion", C.c_int32),
        ("use_adiabatic_focus", C.c_int32),
        ("use_adiabatic_change", C.c_int32),
        ("check_seed_population", C.c_int32),
        ("use_ep_boundary", C.c_int32),
        ("use_boundary_function", C.c_int32),
        ("adiabatic_focus_alg", C.c_int32),
        ("adiabatic_change_alg", C.c_int32),
        ("damp_cooling", C.c_double),
        ("dsh_min", C.c_double),
        ("mfp_type", C.c_int32),
        ("lamo", C.c_double),
        ("mfp_radial_power", C.c_double),
        ("mfp_b_power", C.c_double),
        ("mhd_bs_au", C.c_double),
        ("bf_amplitude", C.c_double),
        ("bf_xi", C.c_double),
        ("bf_gamma", C.c_double),
        ("bf_beta", C.c_double),
        ("bf_ecutoff", C.c_double),
        ("bf_r0", C.c_double),
        ("mhd_us", C.c_double),
        ("mhd_ns_au", C.c_double),
        ("omega_sun", C.c_double),
        ("ideal_shock", C.c_int32),
        ("ideal_shock_sharpness", C.c_double),
        ("ideal_shock_scale_length", C.c_double),
        ("ideal_shock_jump", C.c_double),
        ("ideal_shock_falloff", C.c_double),
        ("ideal_shock_speed", C.c_double),
        ("ideal_shock_init_time", C.c_double),
        ("ideal_shock_theta", C.c_double),
        ("ideal_shock_phi", C.c_double),
        ("ideal_shock_width", C.c_double),
        ("max_subcycles", C.c_int32),
        ("stream_variant", C.c_int32),
    ]


class DriftParams(C.Structure):
    """eprem_drift_params_t"""
    _fields_ = [("lnpmin", C.c_double), ("charge", C.c_double), ("mass", C.c_double)]


class Grids(C.Structure):
    _fields_ = [
        ("egrid", C.POINTER(C.c_double)),
        ("vgrid", C.POINTER(C.c_double)),
        ("vgrid_i", C.POINTER(C.c_double)),
        ("mugrid", C.POINTER(C.c_double)),
        ("rigidity", C.POINTER(C.c_double)),
        ("dlnp", C.c_double),
        ("dmu", C.c_double),
    ]


class EpStats(C.Structure):
    _fields_ = [
        ("max_subcycles_change", C.c_int32),
        ("max_subcycles_focusing", C.c_int32),
        ("max_substeps_stream", C.c_int32),
        ("pad", C.c_int32),
        ("min_tau", C.c_double),
        ("stream_cell_subcycles", C.c_double),
        ("focus_cell_subcycles", C.c_double),
        ("change_cell_subcycles", C.c_double),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_ if name != "pad"}


KERNEL_KINDS = ["geometry", "stream", "node", "seed_check", "mhd", "move", "flux", "convert",
                "shell"]


class KernelTime(C.Structure):
    _fields_ = [("launches", C.c_int32), ("pad", C.c_int32), ("total_ms", C.c_double)]


# enum eprem_node_field, in header order
NODE_FIELDS = [
    "RX", "RY", "RZ", "RMAG",
    "BMAG", "DLNB", "DLNN", "DUPAR",
    "DS", "BMAG_PLUS", "BMAG_MINUS",
    "BR", "BTHETA", "BPHI",
    "VR", "VTHETA", "VPHI",
    "VMAG", "DENSITY", "DIVV",
    "BVEC_X", "BVEC_Y", "BVEC_Z",
    "VVEC_X", "VVEC_Y", "VVEC_Z",
    "BMAG_OLD", "DENSITY_OLD",
    "VSPH_OLD_R", "VSPH_OLD_THETA", "VSPH_OLD_PHI",
    "DS_OLD",
    "ROLD_X", "ROLD_Y", "ROLD_Z",
    "ROLDER_X", "ROLDER_Y", "ROLDER_Z",
]
NODE = {name: i for i, name in enumerate(NODE_FIELDS)}
NODE_NFIELDS = len(NODE_FIELDS)
NODE_MASK_ALL = (1 << NODE_NFIELDS) - 1


def node_mask(*names):
    m = 0
    for n in names:
        m |= 1 << NODE[n]
    return m


# The node fields the energetic-particle update reads and writes.
EP_INPUT_MASK = node_mask("RX", "RY", "RZ", "RMAG", "BMAG", "DLNB", "DLNN", "DUPAR")
EP_OUTPUT_MASK = node_mask("DS", "BMAG_PLUS", "BMAG_MINUS")


# MAS coupling (include/eprem_gpu.h): Bp, Bt, Br, Vp, Vt, Vr, rho
MAS_NFIELDS = 7
MAS_FIELDS = ["Bp", "Bt", "Br", "Vp", "Vt", "Vr", "rho"]


class MasSlice(C.Structure):
    _fields_ = [
        ("dims", (C.c_int32 * 3) * MAS_NFIELDS),
        ("mesh", (C.POINTER(C.c_float) * 3) * MAS_NFIELDS),
        ("data", C.POINTER(C.c_float) * MAS_NFIELDS),
    ]


class MasParams(C.Structure):
    _fields_ = [
        ("radial_max", C.c_double),
        ("v_min", C.c_double),
        ("cor_rotate_fake", C.c_int32),
        ("rotate_solution", C.c_int32),
        ("max_slices", C.c_int32),
        ("pad", C.c_int32),
    ]
