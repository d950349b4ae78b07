"""Reader for the named-array files written by oracle/ref_harness (format TFG1)."""
import struct

import numpy as np

_TYPES = {b"d": np.float64, b"l": np.int64, b"i": np.int32}


def read_tfg(path):
    out = {}
    with open(path, "rb") as f:
        if f.read(4) != b"TFG1":
            raise ValueError(f"{path}: not a TFG1 file")
        while True:
            head = f.read(4)
            if not head:
                break
            (ln,) = struct.unpack("<I", head)
            name = f.read(ln).decode()
            typ = f.read(1)
            (n,) = struct.unpack("<Q", f.read(8))
            dt = np.dtype(_TYPES[typ])
            out[name] = np.frombuffer(f.read(n * dt.itemsize), dtype=dt).copy()
    return out
