"""Coefficient files: a binary checkpoint format and the reference's text dump.

Binary checkpoint (little-endian, self-describing, used to save and resume a
run and to exchange states with CPU tools):

    offset  size  field
    0       8     magic  b"ADSGCKP1"
    8       4     ndim (int32)
    12      12    dofs per direction (3 x int32, 1 for absent directions)
    24      12    degree per direction (3 x int32, 0 for absent)
    36      4     step (int32)
    40      8     dt (float64)
    48      8     t (float64)
    56      ...   coefficients, float64, x-fastest (u[i + nx*(j + ny*k)])

Text dump: the "i j value" lines the reference's examples write and its
ads-error tool reads back (tools/error.cpp:16-30); 3D adds a k column.
"""
from __future__ import annotations

import struct

import numpy as np

MAGIC = b"ADSGCKP1"
_HEADER = struct.Struct("<8si3i3iidd")


def save(path: str, u: np.ndarray, shape, degrees=(), step: int = 0, dt: float = 0.0, t: float = 0.0) -> None:
    u = np.ascontiguousarray(u, dtype="<f8").ravel()
    shape = list(shape)
    if not 1 <= len(shape) <= 3 or int(np.prod(shape)) != u.size:
        raise ValueError("shape must have 1..3 entries whose product is the number of coefficients")
    dims = shape + [1] * (3 - len(shape))
    degs = list(degrees) + [0] * (3 - len(degrees))
    with open(path, "wb") as f:
        f.write(_HEADER.pack(MAGIC, len(shape), *dims, *degs, int(step), float(dt), float(t)))
        f.write(u.tobytes())


def load(path: str):
    """Returns (u, info) with info = {ndim, shape, degrees, step, dt, t}."""
    with open(path, "rb") as f:
        head = f.read(_HEADER.size)
        if len(head) != _HEADER.size:
            raise ValueError(f"{path}: truncated header")
        magic, ndim, d0, d1, d2, p0, p1, p2, step, dt, t = _HEADER.unpack(head)
        if magic != MAGIC:
            raise ValueError(f"{path}: not an ADS checkpoint")
        if not 1 <= ndim <= 3:
            raise ValueError(f"{path}: bad ndim {ndim}")
        shape = (d0, d1, d2)[:ndim]
        n = int(np.prod(shape))
        u = np.frombuffer(f.read(8 * n), dtype="<f8")
        if u.size != n:
            raise ValueError(f"{path}: truncated data ({u.size} of {n} coefficients)")
    info = {"ndim": ndim, "shape": shape, "degrees": (p0, p1, p2)[:ndim], "step": step, "dt": dt, "t": t}
    return u.astype(np.float64), info


def write_text(path: str, u: np.ndarray, shape) -> None:
    """'i j value' (or 'i j k value') per coefficient, as the reference writes."""
    shape = list(shape)
    U = np.asarray(u, np.float64).reshape(shape[::-1])
    with open(path, "w") as f:
        for idx in np.ndindex(*shape[::-1]):
            ijk = idx[::-1]
            f.write(" ".join(str(v) for v in ijk) + f" {float(U[idx])!r}\n")


def read_text(path: str, shape) -> np.ndarray:
    shape = list(shape)
    U = np.zeros(shape[::-1])
    with open(path) as f:
        for line in f:
            parts = line.split()
            if len(parts) != len(shape) + 1:
                continue
            ijk = [int(v) for v in parts[:-1]]
            U[tuple(ijk[::-1])] = float(parts[-1])
    return np.ascontiguousarray(U.ravel())
