"""Reader for the tagged binary container written by oracle/ref_driver.cpp.

Layout per array: [u32 name length][name][dtype char 'd'|'i'|'q'][u32 ndim][u64 dims...][raw little-endian data].
"""
import struct

import numpy as np

_DT = {"d": np.float64, "i": np.int32, "q": np.int64}


def read_container(path):
    out = {}
    with open(path, "rb") as fh:
        buf = fh.read()
    off = 0
    while off < len(buf):
        (nl,) = struct.unpack_from("<I", buf, off)
        off += 4
        name = buf[off:off + nl].decode()
        off += nl
        dt = chr(buf[off])
        off += 1
        (nd,) = struct.unpack_from("<I", buf, off)
        off += 4
        dims = struct.unpack_from("<%dQ" % nd, buf, off)
        off += 8 * nd
        dtype = np.dtype(_DT[dt])
        count = int(np.prod(dims)) if nd else 1
        arr = np.frombuffer(buf, dtype=dtype, count=count, offset=off).reshape(dims).copy()
        off += count * dtype.itemsize
        out[name] = arr
    return out
