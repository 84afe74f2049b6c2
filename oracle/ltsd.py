"""Test infrastructure: reader/writer for the LTSD dump container used by the oracle tools.

Layout: b"LTSD", then records of
  u32 name_len | name | dtype char (f=f32, d=f64, i=i32, u=u32, q=u64) | u64 count | data.
"""
import struct

import numpy as np

_DT = {"f": np.float32, "d": np.float64, "i": np.int32, "u": np.uint32, "q": np.uint64}
_CH = {np.dtype(v).str: k for k, v in _DT.items()}


def read(path):
    with open(path, "rb") as f:
        buf = f.read()
    if buf[:4] != b"LTSD":
        raise ValueError(f"{path}: not an LTSD file")
    out, pos = {}, 4
    while pos < len(buf):
        (nl,) = struct.unpack_from("<I", buf, pos)
        pos += 4
        name = buf[pos:pos + nl].decode()
        pos += nl
        dt = _DT[chr(buf[pos])]
        pos += 1
        (cnt,) = struct.unpack_from("<Q", buf, pos)
        pos += 8
        nb = cnt * np.dtype(dt).itemsize
        out[name] = np.frombuffer(buf, dtype=dt, count=cnt, offset=pos).copy()
        pos += nb
    return out


def write(path, arrays):
    with open(path, "wb") as f:
        f.write(b"LTSD")
        for name, a in arrays.items():
            a = np.ascontiguousarray(a)
            ch = _CH[a.dtype.str]
            nb = name.encode()
            f.write(struct.pack("<I", len(nb)) + nb + ch.encode() + struct.pack("<Q", a.size))
            f.write(a.tobytes())
