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
