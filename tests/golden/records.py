"""Reader for the flat record files written by golden_driver.cpp.

Each record: u32 name length, name bytes (ASCII), u64 count, count doubles.
"""
import struct

import numpy as np


def read_records(path):
    out = {}
    with open(path, "rb") as fp:
        data = fp.read()
    pos = 0
    while pos < len(data):
        (n,) = struct.unpack_from("<I", data, pos)
        pos += 4
        name = data[pos:pos + n].decode("ascii")
        pos += n
        (c,) = struct.unpack_from("<Q", data, pos)
        pos += 8
        out[name] = np.frombuffer(data, dtype="<f8", count=c, offset=pos).copy()
        pos += 8 * c
    return out
