"""Reader for the record files written by oracle/ref_harness/lfdem_ref_harness.cpp.

Each file is a sequence of records: uint32 name length, name bytes, one type
byte ('d' float64 or 'i' int32), uint64 element count, then the data.
"""
import struct

import numpy as np


def read_records(path):
    out = {}
    with open(path, "rb") as f:
        data = f.read()
    o = 0
    while o < len(data):
        (ln,) = struct.unpack_from("<I", data, o); o += 4
        name = data[o:o + ln].decode(); o += ln
        t = chr(data[o]); o += 1
        (cnt,) = struct.unpack_from("<Q", data, o); o += 8
        dt = np.float64 if t == "d" else np.int32
        nbytes = cnt * np.dtype(dt).itemsize
        out[name] = np.frombuffer(data, dtype=dt, count=cnt, offset=o).copy()
        o += nbytes
    return out
