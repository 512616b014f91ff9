"""Checkpoint files of the SIMP loop's state (x, xPhys, U and the iteration
count), so that a loop can stop and resume bit for bit
(``VoxelSolver.TopOpti_GlobalVolumeConstraint(..., return_state=True)`` /
``resume=state``).

The reference's porous-infill loop writes its restart state as NIfTI volumes
(src/TopOpti_LocalVolumeConstraint.m:318-334) and its global loop cannot
resume.  Here the state goes to one raw little-endian binary file:

    bytes 0-7    magic b"SGLDCKPT"
    uint32       format version (1)
    uint32       iterations done (loop)
    uint64       numElements
    uint64       numDOFs
    float64[numElements]  x      (design variables)
    float64[numElements]  xPhys  (filtered design)
    float64[numDOFs]      U      (displacement, compact node-major order)
"""
from __future__ import annotations

import struct

import numpy as np

MAGIC = b"SGLDCKPT"
VERSION = 1
_HEADER = struct.Struct("<8sIIQQ")


def save(path: str, state: dict) -> None:
    x = np.ascontiguousarray(state["x"], dtype="<f8").reshape(-1)
    xp = np.ascontiguousarray(state["xPhys"], dtype="<f8").reshape(-1)
    U = np.ascontiguousarray(state["U"], dtype="<f8").reshape(-1)
    if x.size != xp.size:
        raise ValueError("x and xPhys must have the same length")
    with open(path, "wb") as f:
        f.write(_HEADER.pack(MAGIC, VERSION, int(state["loop"]), x.size, U.size))
        f.write(x.tobytes())
        f.write(xp.tobytes())
        f.write(U.tobytes())


def load(path: str) -> dict:
    with open(path, "rb") as f:
        magic, version, loop, ne, nd = _HEADER.unpack(f.read(_HEADER.size))
        if magic != MAGIC or version != VERSION:
            raise ValueError(f"{path}: not an SGLD checkpoint (version {VERSION})")
        x = np.frombuffer(f.read(8 * ne), dtype="<f8").astype(np.float64)
        xp = np.frombuffer(f.read(8 * ne), dtype="<f8").astype(np.float64)
        U = np.frombuffer(f.read(8 * nd), dtype="<f8").astype(np.float64)
        if x.size != ne or xp.size != ne or U.size != nd:
            raise ValueError(f"{path}: truncated checkpoint")
    return {"loop": int(loop), "x": x, "xPhys": xp, "U": U}
