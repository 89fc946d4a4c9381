"""Text digest of EPREM observer output captured by oracle/ref_shims.c.

TEST INFRASTRUCTURE ONLY.  The reference's testsuite stores, per run, a text
digest of its netCDF observer files (bin/epremdigest.py in the reference; the
goldens are testsuite/<case>/reference/eprem_digest.txt) and passes a run when
its digest is identical.  This module makes the same text from the `.cap`
files the netCDF capture writes, so a run of the reference driver here (or of
the driver with the GPU / oracle path dropped in) is compared with the goldens
line by line.

The digest format follows the reference script (bin/epremdigest.py:33-120),
restated here:
  * one `file <name>` line per obs*.nc, in sorted order, then its variables in
    sorted name order, 0-d variables skipped;
  * per variable: `shape=<numpy shape> dtype=<numpy dtype>`, the global min,
    max, mean, sum and rms (NaN-ignoring numpy reductions) each rounded to 6
    significant figures, and the SHA-256 of the variable's little-endian
    bytes;
  * values as the netCDF4 Python reader returns them: packed values times
    `scale_factor` (plus `add_offset`) when those attributes are set.
"""
import glob
import hashlib
import math
import os
import struct

import numpy as np

_TYPES = {4: np.dtype("<i4"), 5: np.dtype("<f4"), 6: np.dtype("<f8")}


def read_capture(path):
    """Variables of one `.cap` file: {name: (array, scale or None, offset or None)}."""
    with open(path, "rb") as fh:
        raw = fh.read()
    if raw[:8] != b"EPCAP1\n\0":
        raise ValueError(f"{path}: not a netCDF capture")
    pos = 8
    (nvars,) = struct.unpack_from("<i", raw, pos)
    pos += 4
    out = {}
    for _ in range(nvars):
        (nl,) = struct.unpack_from("<i", raw, pos)
        pos += 4
        name = raw[pos:pos + nl].decode()
        pos += nl
        t, nd = struct.unpack_from("<ii", raw, pos)
        pos += 8
        shape = struct.unpack_from("<" + "q" * nd, raw, pos)
        pos += 8 * nd
        hs, scale = struct.unpack_from("<id", raw, pos)
        pos += 12
        ho, offset = struct.unpack_from("<id", raw, pos)
        pos += 12
        dt = _TYPES[t]
        n = int(np.prod(shape)) if nd else 1
        arr = np.frombuffer(raw, dtype=dt, count=n, offset=pos).reshape(shape).copy()
        pos += n * dt.itemsize
        out[name] = (arr, scale if hs else None, offset if ho else None)
    return out


def unpacked(arr, scale, offset):
    """The values a netCDF4 reader returns for a variable with these attributes."""
    if scale is None and offset is None:
        return arr
    s = np.float64(scale if scale is not None else 1.0)
    o = np.float64(offset if offset is not None else 0.0)
    if scale is not None and offset is not None:
        if o != 0.0 or s != 1.0:
            return arr * s + o
        return arr.astype(np.float64)
    if scale is not None:
        return arr * s if s != 1.0 else arr.astype(np.float64)
    return arr + o if o != 0.0 else arr.astype(np.float64)


def sig6(x):
    """x rounded to 6 significant figures, printed with %.6g."""
    x = float(x)
    if math.isnan(x):
        return "nan"
    if math.isinf(x):
        return "inf" if x > 0 else "-inf"
    if x == 0.0:
        return "0.0"
    digits = 6 - int(math.floor(math.log10(abs(x)))) - 1
    return "%.6g" % round(x, digits)


def var_lines(name, a):
    a = np.asarray(a)
    lines = [f"var {name}", f"  shape={a.shape} dtype={a.dtype}"]
    f = np.asarray(a, dtype="float64")
    if f.size == 0:
        lines.append("  min=nan max=nan mean=nan sum=0.0 rms=nan")
    else:
        with np.errstate(invalid="ignore", divide="ignore"):
            stats = (np.nanmin(f), np.nanmax(f), np.nanmean(f), np.nansum(f),
                     np.sqrt(np.nanmean(f * f)))
        lines.append("  min=%s max=%s mean=%s sum=%s rms=%s" % tuple(sig6(v) for v in stats))
    b = a.astype("<" + a.dtype.str[1:]) if a.dtype.kind == "f" else a
    lines.append("  sha256=" + hashlib.sha256(b.tobytes()).hexdigest())
    return lines


def digest_run(rundir, prefix="obs"):
    """Digest text of every <prefix>*.nc capture in rundir (granularity=global;
    prefix "flux" for the streamFluxOutput files, src/unifiedOutput.c:115-122)."""
    lines = ["# eprem_digest granularity=global"]
    for cap in sorted(glob.glob(os.path.join(rundir, prefix + "*.nc.cap"))):
        lines.append("file " + os.path.basename(cap)[:-4])
        vs = read_capture(cap)
        for name in sorted(vs):
            arr, scale, offset = vs[name]
            if arr.ndim == 0:
                continue
            lines.extend(var_lines(name, unpacked(arr, scale, offset)))
    lines.append("")
    return "\n".join(lines)


def parse_digest(text):
    """{(file, var): {"shape":..., "stats":..., "sha256":...}} of a digest text."""
    out, fname, var = {}, None, None
    for ln in text.splitlines():
        if ln.startswith("file "):
            fname = ln[5:].strip()
        elif ln.startswith("var "):
            var = ln[4:].strip()
            out[(fname, var)] = {}
        elif ln.startswith("  shape="):
            out[(fname, var)]["shape"] = ln.strip()
        elif ln.startswith("  min="):
            out[(fname, var)]["stats"] = ln.strip()
        elif ln.startswith("  sha256="):
            out[(fname, var)]["sha256"] = ln.strip()[7:]
    return out
