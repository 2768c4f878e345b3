"""qmc flat model files, the reference's on-disk scene format: prefix.pnt,
prefix.nrm, prefix.col hold float3 per point and prefix.rng int triples
(first point index of a column, x index, y index) — written by qmc
(src/qubatron/qmc.c:275-327), read by model_load_flat
(src/qubatron/model.c:53-111).

read_flat goes through the library's host reader (qbc_flat_read);
OctreeGLC.load_flat reads, builds the tree on the GPU and uploads the model
(qbc_load_flat). write_flat stores arrays in the same format.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import check

EXTS = (".pnt", ".col", ".nrm", ".rng")


def paths(prefix: str):
    """(pnt, col, nrm, rng) paths of a flat model, in qbc_flat_read's order."""
    return tuple(prefix + e for e in EXTS)


def write_flat(prefix: str, points, normals, colors, ranges=None) -> None:
    """Write float3 arrays (and optional int range triples) as qmc flat files."""
    for arr, ext in ((points, ".pnt"), (normals, ".nrm"), (colors, ".col")):
        np.ascontiguousarray(arr, np.float32).reshape(-1, 3).tofile(prefix + ext)
    np.ascontiguousarray(ranges if ranges is not None else np.zeros(0), np.int32).reshape(-1).tofile(prefix + ".rng")


def read_flat(prefix: str, ranges: bool = True) -> dict:
    """qbc_flat_read: point count from the .pnt size, the three float3 arrays,
    the range ints."""
    lib = _lib.load()
    p = [s.encode() for s in paths(prefix)]
    rng_path = p[3] if ranges else None
    n, nr = C.c_int64(), C.c_int64()
    check(lib.qbc_flat_read(p[0], p[1], p[2], rng_path, None, None, None, 0, C.byref(n), None, 0, C.byref(nr)))
    out = {k: np.zeros((n.value, 3), np.float32) for k in ("points", "colors", "normals")}
    rng = np.zeros(max(nr.value, 1), np.int32)
    f = _lib.c_float_p
    check(lib.qbc_flat_read(p[0], p[1], p[2], rng_path, out["points"].ctypes.data_as(f),
                            out["colors"].ctypes.data_as(f), out["normals"].ctypes.data_as(f), n.value, C.byref(n),
                            rng.ctypes.data_as(C.POINTER(C.c_int32)), rng.size, C.byref(nr)))
    out["ranges"] = rng[:nr.value]
    return out
