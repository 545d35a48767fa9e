"""Test infrastructure only: reader/writer for the record files exchanged with
oracle/ref_driver (the reference-linked golden-vector driver).

Record layout: char name[32]; char kind ('d' f64 | 'i' i32); int64 count; data.
"""
import struct

import numpy as np


def write_bag(path, records):
    with open(path, "wb") as f:
        for name, arr in records.items():
            a = np.asarray(arr)
            if a.dtype.kind == "f":
                kind, a = b"d", np.ascontiguousarray(a, dtype="<f8").ravel()
            else:
                kind, a = b"i", np.ascontiguousarray(a, dtype="<i4").ravel()
            nb = name.encode()[:31].ljust(32, b"\0")
            f.write(nb + kind + struct.pack("<q", a.size))
            f.write(a.tobytes())


def read_bag(path):
    out = {}
    with open(path, "rb") as f:
        while True:
            head = f.read(41)
            if len(head) < 41:
                break
            name = head[:32].rstrip(b"\0").decode()
            kind = head[32:33]
            (n,) = struct.unpack("<q", head[33:41])
            dt = "<f8" if kind == b"d" else "<i4"
            out[name] = np.frombuffer(f.read(n * np.dtype(dt).itemsize), dtype=dt).copy()
    return out
