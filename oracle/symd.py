"""ORACLE - test infrastructure only.  Named-array archive ("SYMD") used to
exchange inputs and outputs with oracle/ref_harness.cpp: "SYMD", then records
of u32 name length, name, u8 type ('d' f64, 'i' i32, 'u' u8, 'q' u64),
u64 count, payload."""
from __future__ import annotations

import struct

import numpy as np

_TYPES = {"d": np.float64, "i": np.int32, "u": np.uint8, "q": np.uint64}
_CODES = {np.dtype(v): k for k, v in _TYPES.items()}


def write(path, arrays: dict):
    with open(path, "wb") as f:
        f.write(b"SYMD")
        for name, value in arrays.items():
            if isinstance(value, str):
                arr = np.frombuffer(value.encode(), np.uint8)
            else:
                arr = np.ascontiguousarray(np.asarray(value)).reshape(-1)
                if arr.dtype == np.bool_:
                    arr = arr.astype(np.uint8)
                if arr.dtype not in _CODES:
                    arr = arr.astype(np.float64 if arr.dtype.kind == "f" else np.int32)
            code = _CODES[arr.dtype]
            nb = name.encode()
            f.write(struct.pack("<I", len(nb)) + nb + code.encode() + struct.pack("<Q", arr.size))
            f.write(arr.tobytes())


def read(path) -> dict:
    data = open(path, "rb").read()
    if data[:4] != b"SYMD":
        raise ValueError(f"{path}: not a SYMD archive")
    out, at = {}, 4
    while at < len(data):
        (n,) = struct.unpack_from("<I", data, at)
        at += 4
        name = data[at:at + n].decode()
        at += n
        code = chr(data[at])
        at += 1
        (count,) = struct.unpack_from("<Q", data, at)
        at += 8
        dt = np.dtype(_TYPES[code])
        out[name] = np.frombuffer(data, dt, count, at).copy()
        at += count * dt.itemsize
    return out


def text(arrays: dict, name: str) -> str:
    return bytes(arrays[name]).decode()
