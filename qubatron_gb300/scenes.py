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
# house scale: 3 floors x 6 rooms, 40 boxes and 20 spheres per room on average
SPECS["house90m"] = SceneSpec(_lib.SCENE_HOUSE, 90_000_000, 5, 720, (20.0, 300.0), 360, (10.0, 150.0), 0.05)
# scenes this large are built on the GPU (qbc_build_tree), not by the host producer
GPU_BUILD_POINTS = 30_000_000


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


def make_scene(spec, nodes: bool = True) -> Scene:
    """Points, attributes and (unless nodes is False) the host-built node
    array of a spec; without nodes, Scene.nodes is None and the caller builds
    the tree on the GPU from Scene.points."""
    if isinstance(spec, str):
        spec = SPECS[spec]
    pts, nrm, col = generate_points(spec)
    arr = build_octree(pts, spec.basesize, spec.levels) if nodes else None
    return Scene(spec, pts, nrm, col, arr)


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
    sizes: List = None        # per-view (width, height) when views differ in size
    character: int = 0        # points of a dynamic character re-skinned every frame
    character_root: tuple = (900.0, 500.0, 1100.0)
    train_poses: List = None  # poses whose plain shadow walks train the occluder-proposal network
    train_size: tuple = (960, 720)


def aim(pos, target):
    """(yaw, pitch) that point the camera of octree_fsh.c:406-413 from pos at
    target: the unrotated ray looks down -z, yaw turns it towards +x, pitch up."""
    dx, dy, dz = (target[i] - pos[i] for i in range(3))
    return (float(np.float32(math.atan2(dx, -dz))), float(np.float32(math.atan2(dy, math.hypot(dx, dz)))), 0.0)


def batch_views(seed: int, n: int, target=(960.0, 700.0, 1150.0)):
    """n views with sizes drawn uniformly from {320x240, 640x480, 1280x720,
    1920x1080, 3840x2160}, cameras on a seeded ring around target."""
    rng = _SplitMix(seed)
    choices = [(320, 240), (640, 480), (1280, 720), (1920, 1080), (3840, 2160)]
    sizes, poses = [], []
    for _ in range(n):
        sizes.append(choices[min(4, int(rng.uniform(0.0, 5.0)))])
        ang = rng.uniform(0.0, 2.0 * math.pi)
        r = rng.uniform(450.0, 750.0)
        pos = (float(np.float32(target[0] + r * math.sin(ang))), float(np.float32(rng.uniform(250.0, 1000.0))),
               float(np.float32(target[2] + r * math.cos(ang))))
        poses.append((pos, aim(pos, target)))
    return sizes, poses


WORKLOADS = {
    "floor1m_640x480": Workload("floor1m_640x480", "floor1m", 640, 480, [FLOOR_POSE]),
    "room20m_1920x1080x16": Workload("room20m_1920x1080x16", "room20m", 1920, 1080, spline_poses(1002, 16)),
    "room5m_1920x1080x1": Workload("room5m_1920x1080x1", "room5m", 1920, 1080, spline_poses(1002, 16)[:1]),
    # the first view of the room20m batch alone: a counter-capture case of
    # the bench's scene (its DRAM traffic is scaled to the 16-view launch)
    "room20m_1920x1080x1": Workload("room20m_1920x1080x1", "room20m", 1920, 1080, spline_poses(1002, 16)[:1]),
}
_b64_sizes, _b64_poses = batch_views(64, 64)
WORKLOADS["floor1m_char2m_mixed_x64"] = Workload("floor1m_char2m_mixed_x64", "floor1m", 0, 0, _b64_poses,
                                                 sizes=_b64_sizes, character=2_000_000)
# the same batch with the occluder-proposal network: trained (untimed) on the
# plain walk's shadow rays of 256 other ring poses at 960x720, the character
# in its first pose
WORKLOADS["floor1m_char2m_mlp_mixed_x64"] = Workload("floor1m_char2m_mlp_mixed_x64", "floor1m", 0, 0, _b64_poses,
                                                     sizes=_b64_sizes, character=2_000_000,
                                                     train_poses=batch_views(3001, 256)[1])
# one 1920x1080 view of the same floor and 2M-point character (camera on the
# ring, aimed at the character): a small case of the two-tree kernel for
# profiling
WORKLOADS["floor1m_char2m_1920x1080x1"] = Workload("floor1m_char2m_1920x1080x1", "floor1m", 1920, 1080,
                                                   batch_views(65, 1, target=(900.0, 500.0, 1100.0))[1],
                                                   character=2_000_000)
# learned occluder proposal on the floor scene: 256 training poses at 960x720
# (about 10^7 logged shadow rays), 16 held-out poses at 1920x1080
WORKLOADS["floor1m_mlp_1920x1080x16"] = Workload("floor1m_mlp_1920x1080x16", "floor1m", 1920, 1080,
                                                 batch_views(3002, 16)[1], train_poses=batch_views(3001, 256)[1])


# house scale: 32 poses on a seeded spline through the ground floor at
# 3840x2160, a 10M-point character standing in a ground-floor room
WORKLOADS["house90m_char10m_3840x2160x32"] = Workload(
    "house90m_char10m_3840x2160x32", "house90m", 3840, 2160,
    spline_poses(1005, 32, lo=(120.0, 150.0, 120.0), hi=(1680.0, 480.0, 1680.0)), character=10_000_000,
    character_root=(900.0, 40.0, 500.0))
# the same frame with the occluder-proposal network retrained on this scene
# (256 training poses of another ground-floor spline at 960x720)
WORKLOADS["house90m_char10m_mlp_3840x2160x32"] = Workload(
    "house90m_char10m_mlp_3840x2160x32", "house90m", 3840, 2160,
    spline_poses(1005, 32, lo=(120.0, 150.0, 120.0), hi=(1680.0, 480.0, 1680.0)), character=10_000_000,
    character_root=(900.0, 40.0, 500.0),
    train_poses=spline_poses(1006, 256, lo=(120.0, 150.0, 120.0), hi=(1680.0, 480.0, 1680.0)))


def train_views(w: Workload, maxlevel: int = LEVELS, basesize: float = BASESIZE):
    """qbc_view per training pose of a workload (empty if it has none)."""
    from .octree_glc import view_setup
    tw, th = w.train_size
    return [view_setup(tw, th, pos, ang, w.lighta, w.quality, maxlevel, basesize, 0,
                       vertical_fov_focal(th, w.fov_deg) if w.fov_deg else 0.0) for pos, ang in (w.train_poses or [])]


def workload_views(w: Workload, maxlevel: int = LEVELS, basesize: float = BASESIZE, view_setup=None):
    """qbc_view per pose: the reference's uniforms with the configured
    vertical field of view. view_setup derives them (default: the library's
    qbc_view_setup; any function with its arguments and struct layout)."""
    if view_setup is None:
        from .octree_glc import view_setup
    sizes = w.sizes or [(w.width, w.height)] * len(w.poses)
    return [view_setup(sw, sh, pos, ang, w.lighta, w.quality, maxlevel, basesize, 0,
                       vertical_fov_focal(sh, w.fov_deg) if w.fov_deg else 0.0)
            for (sw, sh), (pos, ang) in zip(sizes, w.poses)]


# ---------------------------------------------------------------------------
# dynamic character: capsule limbs on a bone chain (the dynamic basecube)
# ---------------------------------------------------------------------------

@dataclass
class Character:
    rest_points: np.ndarray   # (n, 3) float32
    rest_normals: np.ndarray  # (n, 3) float32
    colors: np.ndarray        # (n, 3) float32
    bone: np.ndarray          # (n,) int32, the bone each point moves with
    joints: np.ndarray        # (n_bones + 1, 3) float64 rest joint positions


def _unit_disc(rng, n):
    """n unit vectors in the plane, by rejection (no trigonometry)."""
    out = np.empty((0, 2))
    while out.shape[0] < n:
        u = rng.uniform(-1.0, 1.0, (2 * n, 2))
        r2 = (u * u).sum(1)
        u = u[(r2 > 1e-6) & (r2 <= 1.0)]
        out = np.concatenate([out, u / np.sqrt((u * u).sum(1, keepdims=True))])
    return out[:n]


def _unit_sphere(rng, n):
    out = np.empty((0, 3))
    while out.shape[0] < n:
        u = rng.uniform(-1.0, 1.0, (2 * n, 3))
        r2 = (u * u).sum(1)
        u = u[(r2 > 1e-6) & (r2 <= 1.0)]
        out = np.concatenate([out, u / np.sqrt((u * u).sum(1, keepdims=True))])
    return out[:n]


def make_character(n_points: int, seed: int = 4, n_bones: int = 12, root=(900.0, 500.0, 1100.0),
                   bone_len: float = 40.0, radius: float = 12.0) -> Character:
    """A chain of n_bones capsules (radius, length bone_len) with seeded
    zig-zag rest directions; points uniform on the capsule surfaces, exact
    normals, one colour per limb."""
    rng = np.random.default_rng(seed)
    joints = [np.array(root, np.float64)]
    for b in range(n_bones):
        d = np.array([rng.uniform(-0.4, 0.4), 1.0, rng.uniform(-0.4, 0.4)])
        joints.append(joints[-1] + bone_len * d / np.linalg.norm(d))
    joints = np.array(joints)
    cyl = 2.0 * np.pi * radius * bone_len
    cap = 4.0 * np.pi * radius * radius
    bone = rng.integers(0, n_bones, n_points).astype(np.int32)
    on_cyl = rng.uniform(0.0, cyl + cap, n_points) < cyl
    a = joints[bone]
    axis = joints[bone + 1] - a
    axis_n = axis / np.linalg.norm(axis, axis=1, keepdims=True)
    # an orthonormal frame around each bone axis
    helper = np.where(np.abs(axis_n[:, :1]) < 0.9, np.array([[1.0, 0.0, 0.0]]), np.array([[0.0, 1.0, 0.0]]))
    e1 = np.cross(axis_n, helper)
    e1 /= np.linalg.norm(e1, axis=1, keepdims=True)
    e2 = np.cross(axis_n, e1)
    disc = _unit_disc(rng, n_points)
    radial = e1 * disc[:, :1] + e2 * disc[:, 1:]
    t = rng.uniform(0.0, 1.0, (n_points, 1))
    pts = a + axis * t + radius * radial
    nrm = radial.copy()
    sph = _unit_sphere(rng, n_points)
    end = np.where((sph * axis_n).sum(1, keepdims=True) > 0.0, joints[bone + 1], a)
    cap_pts = end + radius * sph
    pts = np.where(on_cyl[:, None], pts, cap_pts)
    nrm = np.where(on_cyl[:, None], nrm, sph)
    limb_col = rng.uniform(0.2, 1.0, (n_bones, 3))
    return Character(pts.astype(np.float32), nrm.astype(np.float32), limb_col[bone].astype(np.float32), bone,
                     joints)


def _rot(axis: int, ang: float) -> np.ndarray:
    c, s = math.cos(ang), math.sin(ang)
    if axis == 0:
        return np.array([[1, 0, 0], [0, c, -s], [0, s, c]])
    return np.array([[c, -s, 0], [s, c, 0], [0, 0, 1]])


def pose_bones(ch: Character, frame: int, seed: int = 9, max_deg: float = 15.0) -> np.ndarray:
    """Bone transforms of one frame: every bone turns by uniform +-max_deg
    about its local x and z axes, accumulated down the chain (forward
    kinematics). Returns (n_bones, 12) float32: row-major R, then t with
    p' = R p + t."""
    rng = np.random.default_rng([seed, frame])
    n_bones = ch.joints.shape[0] - 1
    out = np.zeros((n_bones, 12), np.float64)
    R = np.eye(3)
    j = ch.joints[0].copy()
    lim = math.radians(max_deg)
    for b in range(n_bones):
        R = R @ _rot(0, rng.uniform(-lim, lim)) @ _rot(2, rng.uniform(-lim, lim))
        t = j - R @ ch.joints[b]
        out[b, :9] = R.reshape(-1)
        out[b, 9:] = t
        j = j + R @ (ch.joints[b + 1] - ch.joints[b])
    return out.astype(np.float32)


def skin_reference(ch: Character, bones: np.ndarray):
    """Host skinning in float32 with the operation order of qbc_skin_rigid:
    ((r0 x + r1 y) + r2 z) + t."""
    m = bones[ch.bone]
    p, n = ch.rest_points, ch.rest_normals
    x, y, z = p[:, 0], p[:, 1], p[:, 2]
    px = m[:, 0] * x + m[:, 1] * y + m[:, 2] * z + m[:, 9]
    py = m[:, 3] * x + m[:, 4] * y + m[:, 5] * z + m[:, 10]
    pz = m[:, 6] * x + m[:, 7] * y + m[:, 8] * z + m[:, 11]
    a, b, c = n[:, 0], n[:, 1], n[:, 2]
    nx = m[:, 0] * a + m[:, 1] * b + m[:, 2] * c
    ny = m[:, 3] * a + m[:, 4] * b + m[:, 5] * c
    nz = m[:, 6] * a + m[:, 7] * b + m[:, 8] * c
    return np.stack([px, py, pz], 1).astype(np.float32), np.stack([nx, ny, nz], 1).astype(np.float32)
