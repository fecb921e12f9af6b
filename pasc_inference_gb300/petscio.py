"""PETSc binary vector files, the format the reference reads and writes for signals, gamma
and results (GeneralVector::load_global / save_binary through PETSc VecLoad/VecView):
int32 big-endian class id 1211214, int32 big-endian length n, n big-endian FP64 values."""
from __future__ import annotations

import struct

import numpy as np

VEC_FILE_CLASSID = 1211214


def load_vec(path: str) -> np.ndarray:
    with open(path, "rb") as f:
        head = f.read(8)
        if len(head) != 8:
            raise ValueError(f"{path}: truncated header")
        cid, n = struct.unpack(">ii", head)
        if cid != VEC_FILE_CLASSID:
            raise ValueError(f"{path}: class id {cid} is not a PETSc Vec ({VEC_FILE_CLASSID})")
        body = f.read(8 * n)
        if len(body) != 8 * n:
            raise ValueError(f"{path}: expected {n} values")
    return np.frombuffer(body, dtype=">f8").astype(np.float64)


def save_vec(path: str, v) -> None:
    v = np.ascontiguousarray(v, dtype=np.float64)
    with open(path, "wb") as f:
        f.write(struct.pack(">ii", VEC_FILE_CLASSID, v.size))
        f.write(v.astype(">f8").tobytes())
