"""Snapshot files of the library (rbc_write_snapshot / rbc_read_snapshot), read
and written with numpy alone.

The layout mirrors the reference's HDF5 snapshots (Navier2D::write,
src/navier/navier.rs:975-1013): datasets "temp/v", "temp/vhat" (complex
spectral arrays as "temp/vhat_re" and "temp/vhat_im"), the same for ux, uy,
pres, the grid "x", "dx", "y", "dy", and the scalars time, ra, pr, nu, kappa.

Binary layout (little-endian): b"RBCSNAP1" | u32 version | u32 ndatasets |
i32 nx, ny, kind, precision | f64 dt, aspect | f64 time, ra, pr, nu, kappa |
ndatasets x (char name[32] | i64 rows, cols | u64 offset, bytes) | data.
"""
from __future__ import annotations

import struct

import numpy as np

MAGIC = b"RBCSNAP1"
_HEAD = struct.Struct("<8sII4i2d5d")
_ENTRY = struct.Struct("<32sqqQQ")


def read_snapshot(path):
    """Return {"params": {...}, "scalars": {...}, "datasets": {name: array}}."""
    with open(path, "rb") as f:
        raw = f.read()
    head = _HEAD.unpack_from(raw, 0)
    magic, version, nd = head[0], head[1], head[2]
    if magic != MAGIC or version != 1:
        raise ValueError(f"{path}: not a snapshot file of this library")
    nx, ny, kind, precision = head[3:7]
    dt, aspect = head[7:9]
    time, ra, pr, nu, kappa = head[9:14]
    datasets = {}
    pos = _HEAD.size
    for _ in range(nd):
        name, rows, cols, offset, nbytes = _ENTRY.unpack_from(raw, pos)
        pos += _ENTRY.size
        name = name.split(b"\0", 1)[0].decode()
        if nbytes != rows * cols * 8 or offset + nbytes > len(raw):
            raise ValueError(f"{path}: inconsistent dataset {name}")
        a = np.frombuffer(raw, dtype="<f8", count=rows * cols, offset=offset).reshape(rows, cols)
        datasets[name] = a[:, 0].copy() if cols == 1 else a.copy()
    return {"params": {"nx": nx, "ny": ny, "kind": kind, "precision": precision, "dt": dt, "aspect": aspect,
                       "ra": ra, "pr": pr},
            "scalars": {"time": time, "ra": ra, "pr": pr, "nu": nu, "kappa": kappa},
            "datasets": datasets}


def write_snapshot(path, params, scalars, datasets):
    """Write a snapshot from numpy arrays (1-D arrays are stored as columns)."""
    names = list(datasets)
    arrays = []
    for n in names:
        a = np.ascontiguousarray(datasets[n], dtype="<f8")
        arrays.append(a.reshape(-1, 1) if a.ndim == 1 else a)
    head_size = _HEAD.size + _ENTRY.size * len(names)
    offsets, off = [], head_size
    for a in arrays:
        offsets.append(off)
        off += a.nbytes
    with open(path, "wb") as f:
        f.write(_HEAD.pack(MAGIC, 1, len(names), int(params["nx"]), int(params["ny"]), int(params["kind"]),
                           int(params.get("precision", 0)), float(params["dt"]), float(params["aspect"]),
                           float(scalars["time"]), float(scalars["ra"]), float(scalars["pr"]),
                           float(scalars["nu"]), float(scalars["kappa"])))
        for n, a, o in zip(names, arrays, offsets):
            f.write(_ENTRY.pack(n.encode()[:31], a.shape[0], a.shape[1], o, a.nbytes))
        for a in arrays:
            f.write(a.tobytes())
