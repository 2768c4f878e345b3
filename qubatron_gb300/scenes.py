"""Seeded synthetic scenes and camera poses for the octree ray-cast path.

The reference's assets (res/*.pnt/.nrm/.col) are not available, so every
workload is a seeded procedural scene with the sizes of the benchmark
configurations: one basecube of side 1800 at octree depth 12, points inserted
with octree.c insert-by-position semantics (octree.c:95-147).

* ``floor1m``  1,000,000 points on a floor plane + 40 boxes (sides 50-400)
               + 20 spheres (radius 30-200), per-primitive RGB, 640x480,
               60 degree vertical field of view, one fixed pose.
* ``room20m``  20,000,000 points on a closed room (floor, 4 walls, ceiling)
               + 200 boxes (20-300) + 100 spheres (10-150), per-primitive RGB
               +-0.05 noise, 1920x1080, 16 poses on a seeded Catmull-Rom spline.

Generation and poses use only +, -, *, / and sqrt (and integer hashing), so
the same seed gives the same bits on every machine.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass
from typing import List, Tuple

import numpy as np

from . import _lib
from ._lib import SceneDesc, check
from .octree import build_octree

BASESIZE = 1800.0
LEVELS = 12


@dataclass
class SceneSpec:
    kind: int
    n_points: int
    seed: int
    n_boxes: int
    box: Tuple[float, float]
    n_spheres: int
    sphere: Tuple[float, float]
    color_noise: float = 0.0
    basesize: float = BASESIZE
    levels: int = LEVELS

    def desc(self) -> SceneDesc:
        d = SceneDesc()
        d.kind = self.kind
        d.levels = self.levels
        d.n_points = self.n_points
        d.seed = self.seed
        d.basesize = self.basesize
        d.n_boxes = self.n_boxes
        d.box_min, d.box_max = self.box
        d.n_spheres = self.n_spheres
        d.sphere_min, d.sphere_max = self.sphere
        d.color_noise = self.color_noise
        return d


SPECS = {
    "floor1m": SceneSpec(_lib.SCENE_FLOOR, 1_000_000, 1, 40, (50.0, 400.0), 20, (30.0, 200.0)),
    "room20m": SceneSpec(_lib.SCENE_ROOM, 20_000_000, 2, 200, (20.0, 300.0), 100, (10.0, 150.0), 0.05),
}
# the room scene at a quarter of the points: a profiling case whose node
# arrays (~0.5 GB) still exceed L2 but keep an ncu capture short
SPECS["room5m"] = SceneSpec(_lib.SCENE_ROOM, 5_000_000, 2, 200, (20.0, 300.0), 100, (10.0, 150.0), 0.05)


@dataclass
class Scene:
    spec: SceneSpec
    points: np.ndarray   # (n, 3) float32
    normals: np.ndarray  # (n, 3) float32
    colors: np.ndarray   # (n, 3) float32
    nodes: np.ndarray    # (m, 12) int32, reference node layout


def generate_points(spec: SceneSpec):
    """Points, normals, colours of a spec, in octree-path order."""
    lib = _lib.load()
    n = spec.n_points
    pts = np.empty((n, 3), np.float32)
    nrm = np.empty((n, 3), np.float32)
    col = np.empty((n, 3), np.float32)
    d = spec.desc()
    check(lib.qbc_scene_generate(C.byref(d), pts.ctypes.data_as(_lib.c_float_p), nrm.ctypes.data_as(_lib.c_float_p),
                                 col.ctypes.data_as(_lib.c_float_p)))
    return pts, nrm, col


def make_scene(spec) -> Scene:
    if isinstance(spec, str):
        spec = SPECS[spec]
    pts, nrm, col = generate_points(spec)
    nodes = build_octree(pts, spec.basesize, spec.levels)
    return Scene(spec, pts, nrm, col, nodes)


def scaled_spec(name: str, n_points: int) -> SceneSpec:
    """The named scene with fewer points (same primitives, same seed)."""
    s = SPECS[name]
    return SceneSpec(s.kind, n_points, s.seed, s.n_boxes, s.box, s.n_spheres, s.sphere, s.color_noise, s.basesize,
                     s.levels)


# ---------------------------------------------------------------------------
# camera poses: (position xyz, angle xy) as float32 values
# ---------------------------------------------------------------------------

class _SplitMix:
    def __init__(self, seed: int):
        self.s = seed & 0xFFFFFFFFFFFFFFFF

    def next(self) -> int:
        self.s = (self.s + 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF
        z = self.s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & 0xFFFFFFFFFFFFFFFF
        return z ^ (z >> 31)

    def uniform(self, a: float, b: float) -> float:
        return a + (b - a) * ((self.next() >> 11) * (1.0 / 9007199254740992.0))


def _catmull_rom(p0, p1, p2, p3, t):
    t2 = t * t
    t3 = t2 * t
    return [0.5 * ((2.0 * b) + (-a + c) * t + (2.0 * a - 5.0 * b + 4.0 * c - d) * t2 + (-a + 3.0 * b - 3.0 * c + d) * t3)
            for a, b, c, d in zip(p0, p1, p2, p3)]


def spline_poses(seed: int, n: int, lo=(300.0, 150.0, 300.0), hi=(1500.0, 700.0, 1500.0)):
    """n poses along a seeded Catmull-Rom spline through 8 control points;
    each control point carries (x, y, z, yaw, pitch)."""
    rng = _SplitMix(seed)
    ctrl = []
    for _ in range(8):
        ctrl.append([rng.uniform(lo[0], hi[0]), rng.uniform(lo[1], hi[1]), rng.uniform(lo[2], hi[2]),
                     rng.uniform(-3.0, 3.0), rng.uniform(-0.4, 0.15)])
    segs = len(ctrl) - 3
    poses = []
    for k in range(n):
        u = segs * k / n
        s = int(u)
        t = u - s
        q = _catmull_rom(ctrl[s], ctrl[s + 1], ctrl[s + 2], ctrl[s + 3], t)
        pos = tuple(float(np.float32(x)) for x in q[:3])
        ang = (float(np.float32(q[3])), float(np.float32(q[4])), 0.0)
        poses.append((pos, ang))
    return poses


FLOOR_POSE = ((903.7, 421.3, 1702.9), (0.0, -0.3, 0.0))


def vertical_fov_focal(height_px: float, fov_deg: float = 60.0) -> float:
    """cfp.z giving a vertical field of view of fov_deg on height_px rows."""
    return float(np.float32((height_px / 2.0) / math.tan(math.radians(fov_deg) / 2.0)))


@dataclass
class Workload:
    name: str
    scene: str
    width: int
    height: int
    poses: List
    lighta: float = 0.0
    quality: int = 10
    fov_deg: float = 60.0


WORKLOADS = {
    "floor1m_640x480": Workload("floor1m_640x480", "floor1m", 640, 480, [FLOOR_POSE]),
    "room20m_1920x1080x16": Workload("room20m_1920x1080x16", "room20m", 1920, 1080, spline_poses(1002, 16)),
    "room5m_1920x1080x1": Workload("room5m_1920x1080x1", "room5m", 1920, 1080, spline_poses(1002, 16)[:1]),
}


def workload_views(w: Workload, maxlevel: int = LEVELS, basesize: float = BASESIZE):
    """qbc_view per pose: the reference's uniforms with the configured
    vertical field of view."""
    from .octree_glc import view_setup
    focal = vertical_fov_focal(w.height, w.fov_deg) if w.fov_deg else 0.0
    return [view_setup(w.width, w.height, pos, ang, w.lighta, w.quality, maxlevel, basesize, 0, focal)
            for pos, ang in w.poses]
