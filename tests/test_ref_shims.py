"""Unit tests of the libraries restated for the reference harness
(oracle/ref_shims.c): the libconfig-syntax reader, the netCDF capture and the
HDF5 reader.  They carry the whole-run testsuite pins, so each is checked on
its own here.  Each check runs in a child process that loads the harness
library (oracle/_ref/libeprem_ref.so, built where the reference tree exists).
"""
import json
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "oracle", "_ref", "libeprem_ref.so")
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle as _orc  # noqa: E402  (the reference tree's location only)

REF = _orc.reference_root() or ""

pytestmark = pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "src")),
                                reason="reference source tree not present")


@pytest.fixture(scope="module", autouse=True)
def harness():
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref",
                           f"REF={REF}"])


def _child(body, cwd):
    """Run `body` (Python) in a child with `lib` the loaded harness library;
    return what it prints as JSON."""
    code = "import ctypes as C, json\nlib = C.CDLL(%r)\n" % LIB + textwrap.dedent(body)
    out = subprocess.check_output([sys.executable, "-c", code], cwd=cwd, text=True)
    return json.loads(out.strip().splitlines()[-1])


CONFIG = r'''
# a comment line
intval = 5;
fltval = 5.0
expval : 1e-3
negint=-7
hexval = 0x1F
bigint = 3000000000
strval = "a" "b\tc"
arr = [1.5, 2.5, -3.0]
intarr = [1, 2]
flag = TRUE
grp = { inner = 2.5; deep = { x = 1; }; };
/* a block
   comment */ after = 3 // trailing comment
'''

LOOKUPS = r'''
class Cfg(C.Structure):
    _fields_ = [("impl", C.c_void_p)]
lib.config_lookup.restype = C.c_void_p
lib.config_lookup.argtypes = [C.POINTER(Cfg), C.c_char_p]
lib.config_setting_get_float_elem.restype = C.c_double
lib.config_setting_get_float_elem.argtypes = [C.c_void_p, C.c_int]
lib.config_setting_length.argtypes = [C.c_void_p]
lib.config_error_text.restype = C.c_char_p
def read(path):
    c = Cfg()
    lib.config_init(C.byref(c))
    ok = lib.config_read_file(C.byref(c), path.encode())
    return c, ok
def geti(c, k):
    v = C.c_int(); ok = lib.config_lookup_int(C.byref(c), k.encode(), C.byref(v)); return [ok, v.value]
def getf(c, k):
    v = C.c_double(); ok = lib.config_lookup_float(C.byref(c), k.encode(), C.byref(v)); return [ok, v.value]
def gets(c, k):
    v = C.c_char_p(); ok = lib.config_lookup_string(C.byref(c), k.encode(), C.byref(v))
    return [ok, v.value.decode() if ok else None]
'''


def test_config_reader_types_and_syntax(tmp_path):
    (tmp_path / "cfg").write_text(CONFIG)
    (tmp_path / "bad").write_text("a = 1;\nb = ;\n")
    (tmp_path / "dup").write_text("a = 1\na = 2\n")
    r = _child(LOOKUPS + r'''
c, ok = read("cfg")
arr = lib.config_lookup(C.byref(c), b"arr")
ia = lib.config_lookup(C.byref(c), b"intarr")
res = dict(ok=ok,
    intval_i=geti(c, "intval"), intval_f=getf(c, "intval"),
    fltval_f=getf(c, "fltval"), fltval_i=geti(c, "fltval"),
    expval=getf(c, "expval"), negint=geti(c, "negint"), hexval=geti(c, "hexval"),
    bigint=geti(c, "bigint"), strval=gets(c, "strval"),
    arr_len=lib.config_setting_length(arr),
    arr=[lib.config_setting_get_float_elem(arr, i) for i in range(4)],
    intarr=[lib.config_setting_get_float_elem(ia, i) for i in range(2)],
    inner=getf(c, "grp.inner"), deep=geti(c, "grp.deep.x"), after=geti(c, "after"),
    missing=geti(c, "nothere"))
b, okb = read("bad")
d, okd = read("dup")
res.update(bad_ok=okb, bad_line=lib.config_error_line(C.byref(b)),
           dup_ok=okd, dup_text=lib.config_error_text(C.byref(d)).decode())
print(json.dumps(res))
''', tmp_path)
    assert r["ok"] == 1
    # integers and floats are kept apart, as libconfig does without auto-conversion
    assert r["intval_i"] == [1, 5] and r["intval_f"][0] == 0
    assert r["fltval_f"] == [1, 5.0] and r["fltval_i"][0] == 0
    assert r["expval"] == [1, 1e-3]
    assert r["negint"] == [1, -7] and r["hexval"] == [1, 31]
    assert r["bigint"][0] == 0  # a 64-bit integer does not fit an int lookup
    assert r["strval"] == [1, "ab\tc"]  # adjacent literals concatenate, escapes decode
    assert r["arr_len"] == 3 and r["arr"] == [1.5, 2.5, -3.0, 0.0]
    assert r["intarr"] == [0.0, 0.0]  # integer elements read as floats give 0
    assert r["inner"] == [1, 2.5] and r["deep"] == [1, 1] and r["after"] == [1, 3]
    assert r["missing"][0] == 0
    assert r["bad_ok"] == 0 and r["bad_line"] == 2
    assert r["dup_ok"] == 0 and "duplicate" in r["dup_text"]


def test_netcdf_capture_writes_what_was_put(tmp_path):
    import digest as D
    _child(r'''
NC_INT, NC_DOUBLE = 4, 6
i = C.c_int
nc = i(); t = i(); n = i(); v = i(); w = i()
assert lib.nc_create(b"x.nc", 0, C.byref(nc)) == 0
lib.nc_def_dim(nc, b"time", C.c_size_t(0), C.byref(t))
lib.nc_def_dim(nc, b"n", C.c_size_t(3), C.byref(n))
dims = (i * 2)(t.value, n.value)
lib.nc_def_var(nc, b"v", NC_DOUBLE, 2, dims, C.byref(v))
lib.nc_def_var(nc, b"w", NC_INT, 1, (i * 1)(n.value), C.byref(w))
lib.nc_put_att_double(nc, v, b"scale_factor", NC_DOUBLE, C.c_size_t(1), (C.c_double * 1)(2.0))
lib.nc_enddef(nc)
sz = C.c_size_t * 2
assert lib.nc_put_vara_double(nc, v, sz(1, 0), sz(1, 3), (C.c_double * 3)(1, 2, 3)) == 0
assert lib.nc_put_vara_int(nc, w, (C.c_size_t * 1)(0), (C.c_size_t * 1)(3), (i * 3)(4, 5, 6)) == 0
pd = C.c_ssize_t * 2
data = (C.c_double * 6)(10, 11, 12, 13, 14, 15)
assert lib.nc_put_varm_double(nc, v, sz(2, 0), sz(1, 3), pd(1, 1), pd(0, 2), data) == 0
assert lib.nc_close(nc) == 0
nc2 = i(); vid = i()
assert lib.nc_open(b"x.nc", 1, C.byref(nc2)) == 0
assert lib.nc_inq_varid(nc2, b"v", C.byref(vid)) == 0 and vid.value == v.value
assert lib.nc_put_var1_double(nc2, vid, sz(0, 1), (C.c_double * 1)(9)) == 0
assert lib.nc_close(nc2) == 0
print(json.dumps({}))
''', tmp_path)
    cap = D.read_capture(str(tmp_path / "x.nc.cap"))
    v, scale, offset = cap["v"]
    fill = 9.9692099683868690e+36
    np.testing.assert_array_equal(v, [[fill, 9, fill], [1, 2, 3], [10, 12, 14]])
    assert scale == 2.0 and offset is None
    np.testing.assert_array_equal(D.unpacked(v, scale, offset)[1], [2, 4, 6])
    w, _, _ = cap["w"]
    assert w.dtype == np.int32 and list(w) == [4, 5, 6]


def test_hdf5_reader_on_a_mas_slice(tmp_path):
    path = os.path.join(REF, "testsuite", "mas_wind", "input", "data", "br001.h5")
    if not os.path.exists(path):
        pytest.skip("MAS testsuite input not present")
    r = _child(r'''
lib.H5Fopen.restype = C.c_longlong
lib.H5Fopen.argtypes = [C.c_char_p, C.c_uint, C.c_longlong]
lib.H5Dopen2.restype = C.c_longlong
lib.H5Dopen2.argtypes = [C.c_longlong, C.c_char_p, C.c_longlong]
lib.H5Dget_type.restype = C.c_longlong; lib.H5Dget_type.argtypes = [C.c_longlong]
lib.H5Dget_space.restype = C.c_longlong; lib.H5Dget_space.argtypes = [C.c_longlong]
lib.H5Sget_simple_extent_npoints.restype = C.c_longlong
lib.H5Sget_simple_extent_npoints.argtypes = [C.c_longlong]
lib.H5Dread.argtypes = [C.c_longlong] * 5 + [C.c_void_p]
f = lib.H5Fopen(%r.encode(), 0, 0)
out = {"file": f >= 0}
for name in ("Data", "dim1", "dim2", "dim3"):
    d = lib.H5Dopen2(f, name.encode(), 0)
    sp = lib.H5Dget_space(d)
    npts = lib.H5Sget_simple_extent_npoints(sp)
    buf = (C.c_float * npts)()
    rc = lib.H5Dread(d, 1, 0, 0, 0, buf)
    out[name] = dict(type=lib.H5Dget_type(d), n=npts, rc=rc, first=buf[0], last=buf[npts - 1])
out["missing"] = lib.H5Dopen2(f, b"NoSuchSet", 0)
out["bad_file"] = lib.H5Fopen(b"/nonexistent.h5", 0, 0)
print(json.dumps(out))
''' % path, tmp_path)
    assert r["file"]
    assert r["Data"] == dict(r["Data"], type=1, rc=0) and r["Data"]["n"] == 4 * 4 * 200
    for name, n in (("dim1", 200), ("dim2", 4), ("dim3", 4)):
        assert r[name]["type"] == 1 and r[name]["rc"] == 0 and r[name]["n"] == n
    assert r["dim1"]["last"] > r["dim1"]["first"] > 0  # radial mesh, increasing
    assert r["missing"] < 0 and r["bad_file"] < 0
