"""Node-array producer: the reference's CPU octree (src/qubatron/octree.c)
on libqbcuda's host side.

``Octree`` keeps the reference layout (12 int32 per node: 8 children, the
model index of the point that created the node, 3 pad; node 0 = root; child 0
= empty) so its ``nodes`` array is uploaded unchanged with
``octree_glc_upload_texbuffer_data``.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import check


class Octree:
    """octree_t: create / reset / insert_point / insert_path / remove_point."""

    def __init__(self, basesize: float = 1800.0, levels: int = 12):
        self._lib = _lib.load()
        h = C.c_void_p()
        check(self._lib.qbc_octree_create(float(basesize), int(levels), C.byref(h)))
        self.handle = h
        self.basesize = float(basesize)
        self.levels = int(levels)

    def __del__(self):
        try:
            if self.handle:
                self._lib.qbc_octree_free(self.handle)
                self.handle = None
        except Exception:
            pass

    def reset(self) -> None:
        """octree_reset (octree.c:89-93)."""
        check(self._lib.qbc_octree_reset(self.handle))

    def insert_points(self, points: np.ndarray, first_index: int = 0) -> None:
        """octree_insert_point (octree.c:95-147) for each point in order."""
        p = np.ascontiguousarray(points, dtype=np.float32).reshape(-1, 3)
        check(self._lib.qbc_octree_insert_points(self.handle, p.ctypes.data_as(_lib.c_float_p), p.shape[0],
                                                 int(first_index)))

    def insert_paths(self, octets: np.ndarray, first_index: int = 0) -> None:
        """octree_insert_path (octree.c:149-180); one row of `levels` octets per point."""
        o = np.ascontiguousarray(octets, dtype=np.int32).reshape(-1, self.levels)
        check(self._lib.qbc_octree_insert_paths(self.handle, o.ctypes.data_as(_lib.c_int32_p), o.shape[0],
                                                int(first_index)))

    def remove_point(self, point) -> tuple:
        """octree_remove_point (octree.c:182-218) -> (model index, parent node),
        (-1, -1) when the point's walk meets an empty link."""
        p = (C.c_float * 3)(*[float(x) for x in point])
        m, o = C.c_int32(-1), C.c_int32(-1)
        check(self._lib.qbc_octree_remove_point(self.handle, p, C.byref(m), C.byref(o)))
        return m.value, o.value

    @property
    def nodes(self) -> np.ndarray:
        """Copy of the node array, shape (len, 12) int32."""
        ptr = _lib.c_int32_p()
        n = C.c_int64()
        check(self._lib.qbc_octree_nodes(self.handle, C.byref(ptr), C.byref(n)))
        if n.value == 0:
            return np.zeros((0, 12), np.int32)
        return np.ctypeslib.as_array(ptr, shape=(n.value, 12)).copy()

    def __len__(self) -> int:
        ptr = _lib.c_int32_p()
        n = C.c_int64()
        check(self._lib.qbc_octree_nodes(self.handle, C.byref(ptr), C.byref(n)))
        return n.value


def build_octree(points: np.ndarray, basesize: float = 1800.0, levels: int = 12) -> np.ndarray:
    """Insert every point in order into a fresh tree; return its node array."""
    t = Octree(basesize, levels)
    t.insert_points(points)
    return t.nodes
