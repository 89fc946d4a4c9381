"""The C ABI without a GPU: the library loads, exports every entry point the
header declares, and the ctypes mirror matches the C layout."""
import ctypes as C
import os
import re

import pytest

from eprem_gb300 import abi, runtime

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "eprem_gpu.h")


def header_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"\b(eprem_gpu_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(runtime.LIB_PATH):
        from eprem_gb300 import build
        build.build()
    return runtime.load_library()


def test_header_declares_what_runtime_binds():
    assert header_functions() == sorted(n for n, _, _ in runtime.EXPORTS)


def test_library_exports_every_declared_symbol(lib):
    for name in header_functions():
        assert hasattr(lib, name), name


def test_last_error_callable_without_gpu(lib):
    assert isinstance(lib.eprem_gpu_last_error(), bytes)


def test_create_rejects_bad_arguments_before_touching_a_device(lib):
    d = abi.Dims(6, 2, 1, 8, 6, abi.EPREM_FP64)  # num_nodes < 3
    p = abi.Params()
    g = abi.Grids()
    h = C.c_void_p()
    rc = lib.eprem_gpu_create(C.byref(d), C.byref(p), C.byref(g), C.byref(h))
    assert rc == abi.EPREM_GPU_ERR_ARG
    d = abi.Dims(6, 10, 2, 8, 6, abi.EPREM_FP64)  # two species
    rc = lib.eprem_gpu_create(C.byref(d), C.byref(p), C.byref(g), C.byref(h))
    assert rc == abi.EPREM_GPU_ERR_UNSUPPORTED
    assert b"species" in lib.eprem_gpu_last_error()


def test_ctypes_layout_matches_c(oracle_lib):
    buf = (C.c_long * 256)()
    n = oracle_lib.lib.orc_abi_layout(buf, 256)
    got = list(buf[:n])
    exp = [C.sizeof(abi.Dims), C.sizeof(abi.Params), C.sizeof(abi.Grids), C.sizeof(abi.EpStats),
           abi.NODE_NFIELDS]
    for cls in (abi.Dims, abi.Params, abi.Grids, abi.EpStats):
        exp += [getattr(cls, f).offset for f, _ in cls._fields_]
    assert got == exp


def test_node_field_enum_matches_header():
    text = open(HEADER).read()
    body = text[text.index("enum eprem_node_field"):text.index("EPREM_NODE_NFIELDS\n")]
    names = re.findall(r"EPREM_NODE_([A-Z_]+)", body)
    assert names == abi.NODE_FIELDS


@pytest.mark.parametrize("nodes,mu,bc,expect", [
    # the precision-at-scale streams: the mirrored kind on one 256-thread CTA
    (1000, 40, True, dict(kind=7, mmax=40, threads=256, npt=4, cluster=1)),
    # the MHD-coupled streams: 128 x 4 in clusters of 3 (1501 slots needed)
    (1500, 40, True, dict(kind=7, mmax=40, threads=128, npt=4, cluster=3)),
    # 1022 nodes: list node 0 may start 3 slots in, so 1025 slots -> a cluster
    (1022, 40, True, dict(kind=7, threads=128, npt=4, cluster=3)),
    (1021, 40, True, dict(kind=7, threads=256, npt=4, cluster=1)),
    # the CPU-runnable size: its own 20 bin, a stream on two warps
    (400, 20, True, dict(kind=7, mmax=20, threads=64, npt=7, cluster=1)),
    # no seed boundary: the packed kind with compile-time guards
    (1000, 40, False, dict(kind=5, mmax=40, threads=256, npt=4, cluster=1)),
    # a mu count between bins: the packed kind with run-time guards
    (600, 28, True, dict(kind=4, mmax=32)),
])
def test_stream_plan_without_a_device(lib, nodes, mu, bc, expect):
    """The streaming kernel chosen for a run's sizes (kind 0, automatic):
    the mirrored kind where M is 20 or 40 and the seed boundary is on,
    otherwise the packed kinds; a cluster holds the stream."""
    got = runtime.plan_stream(nodes, mu, mu // 2, abi.EPREM_FP32, 0, bc)
    for k, v in expect.items():
        assert got[k] == v, (k, got)
    need = nodes + (got["npt"] - 1 if got["kind"] in (6, 7) else 0)
    assert got["slots"] >= need
    assert got["slots"] - need < got["threads"] * got["npt"]  # no idle CTA


def test_stream_plan_refusals(lib):
    # the mirrored kinds need the seed boundary and M = 20 or 40
    with pytest.raises(runtime.EpremGpuError):
        runtime.plan_stream(1000, 40, 20, abi.EPREM_FP32, 7, seed_boundary=False)
    with pytest.raises(runtime.EpremGpuError):
        runtime.plan_stream(1000, 32, 16, abi.EPREM_FP32, 7)
    # the FP64 kernel's shapes are not FP32 variants, and the reverse
    with pytest.raises(runtime.EpremGpuError):
        runtime.plan_stream(1000, 40, 20, abi.EPREM_FP32, 1)
    with pytest.raises(runtime.EpremGpuError):
        runtime.plan_stream(1000, 40, 20, abi.EPREM_FP64, 5)
    # more than 8 CTAs per cluster
    with pytest.raises(runtime.EpremGpuError):
        runtime.plan_stream(100000, 40, 20, abi.EPREM_FP32, 0)
    fp64 = runtime.plan_stream(1000, 40, 20, abi.EPREM_FP64, 0)
    assert fp64["kind"] == 0 and fp64["slots"] >= 1000
