"""ctypes wrapper of the CPU oracle (oracle/_build/libqbo.so) and of the
reference's own octree.c build (oracle/_ref/libqbref.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() as the
checker and by bench.py's CPU-baseline leg. The library under test never
calls it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBQBO = os.path.join(HERE, "_build", "libqbo.so")
LIBREF = os.path.join(HERE, "_ref", "libqbref.so")
# the reference checkout the pinning build compiles from: QB_REFERENCE_ROOT,
# or None (no reference build; the committed golden fixtures still pin)
REFERENCE_ROOT = os.environ.get("QB_REFERENCE_ROOT") or None

f32p = C.POINTER(C.c_float)
i32p = C.POINTER(C.c_int32)
u32p = C.POINTER(C.c_uint32)
u8p = C.POINTER(C.c_uint8)
i64p = C.POINTER(C.c_int64)


class QboTree(C.Structure):
    _fields_ = [("nodes", i32p), ("n_nodes", C.c_int64), ("cbox", u32p), ("box_depth", C.c_int32)]


class QboModel(C.Structure):
    _fields_ = [("col", f32p), ("nrm", f32p), ("n_points", C.c_int64)]


class QboScene(C.Structure):
    _fields_ = [("tree", QboTree * 2), ("model", QboModel * 2)]


class QboView(C.Structure):
    _fields_ = [
        ("camfp", C.c_float * 3), ("light", C.c_float * 3), ("basecube", C.c_float * 4), ("dim", C.c_float * 2),
        ("cfp", C.c_float * 3), ("qz", C.c_float * 4), ("qx", C.c_float * 4), ("ncamlight", C.c_float * 3),
        ("flare_cos", C.c_float), ("coord_scale", C.c_float * 2), ("width_px", C.c_int32),
        ("height_px", C.c_int32), ("maxlevel", C.c_int32), ("shoot", C.c_int32),
    ]

    def to_bytes(self) -> bytes:
        return bytes(memoryview(self).cast("B"))

    @classmethod
    def from_bytes(cls, b: bytes) -> "QboView":
        v = cls()
        C.memmove(C.addressof(v), b, C.sizeof(cls))
        return v


class QboHit(C.Structure):
    _fields_ = [
        ("isp", C.c_float * 4), ("col", C.c_float * 4), ("nrm", C.c_float * 4), ("tlf", C.c_float * 4),
        ("leaf", C.c_int32 * 2), ("model", C.c_int32 * 2), ("status", C.c_int32), ("faces", C.c_int32),
        ("visits", C.c_int32 * 2), ("steps", C.c_int32), ("oob", C.c_int32),
    ]


class QboFrame(C.Structure):
    _fields_ = [("rgba", f32p), ("rgba8", u8p), ("flags", u32p), ("leaf", i32p), ("isp", f32p), ("visits", u32p)]


MISS, LEAF, DISCARD = 0, 1, 2

_qbo = None
_ref = None


def build_oracle() -> str:
    """make -C oracle: compile the restatement (gcc, -ffp-contract=off, OpenMP)."""
    res = subprocess.run(["make", "-s", "-C", HERE], capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + res.stdout + res.stderr)
    return LIBQBO


def build_reference(root: str | None = None) -> str | None:
    """Compile the reference's octree.c into oracle/_ref when its sources exist
    under root (default QB_REFERENCE_ROOT; None when neither is given)."""
    root = root or REFERENCE_ROOT
    if not root or not os.path.isfile(os.path.join(root, "src", "qubatron", "octree.c")):
        return None
    res = subprocess.run([os.path.join(HERE, "build_ref.sh"), root], capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("reference build failed:\n" + res.stdout + res.stderr)
    return LIBREF


def qbo() -> C.CDLL:
    global _qbo
    if _qbo is None:
        if not os.path.exists(LIBQBO):
            build_oracle()
        lib = C.CDLL(LIBQBO)
        lib.qbo_trace.argtypes = [C.POINTER(QboScene), f32p, C.c_int, f32p, f32p, C.POINTER(QboHit)]
        lib.qbo_trace.restype = None
        lib.qbo_render.argtypes = [C.POINTER(QboScene), C.POINTER(QboView), C.POINTER(QboFrame), C.c_int]
        lib.qbo_render.restype = None
        lib.qbo_render_pixels.argtypes = [C.POINTER(QboScene), C.POINTER(QboView), i32p, i32p, C.c_int64,
                                          C.POINTER(QboFrame), C.c_int]
        lib.qbo_render_pixels.restype = None
        lib.qbo_trace_rays.argtypes = [C.POINTER(QboScene), C.POINTER(C.c_float), C.c_int, f32p, f32p, C.c_int64,
                                       i32p, i32p, i32p, i32p, C.c_int]
        lib.qbo_trace_rays.restype = None
        lib.qbo_view_setup.argtypes = [C.c_float, C.c_float, f32p, f32p, C.c_float, C.c_int, C.c_int, C.c_float,
                                       C.c_int, C.c_float, C.POINTER(QboView)]
        lib.qbo_view_setup.restype = None
        lib.qbo_unorm8.argtypes = [C.c_float]
        lib.qbo_unorm8.restype = C.c_uint8
        lib.qbo_insert_point.argtypes = [i32p, i64p, C.c_int64, C.c_float, C.c_int, C.c_int64, f32p, i32p]
        lib.qbo_insert_point.restype = C.c_int
        lib.qbo_insert_path.argtypes = [i32p, i64p, C.c_int64, C.c_int, C.c_int64, i32p]
        lib.qbo_insert_path.restype = C.c_int
        lib.qbo_remove_point.argtypes = [i32p, C.c_float, C.c_int, f32p, i32p, i32p]
        lib.qbo_remove_point.restype = None
        lib.qbo_remove_points.argtypes = [i32p, C.c_float, C.c_int, f32p, C.c_int64, i32p, i32p]
        lib.qbo_remove_points.restype = None
        lib.qbo_point_octets.argtypes = [C.c_float, C.c_int, f32p, i32p]
        lib.qbo_build_boxes.argtypes = [i32p, C.c_int64, u32p]
        lib.qbo_build_boxes.restype = C.c_int32
        lib.qbo_point_octets.restype = None
        lib.qbo_build_tree.argtypes = [f32p, C.c_int64, C.c_float, C.c_int, i32p, C.c_int64]
        lib.qbo_build_tree.restype = C.c_int64
        lib.qbo_scene_generate.argtypes = [C.c_int, C.c_int, C.c_int64, C.c_uint64, C.c_float, C.c_int, C.c_float,
                                           C.c_float, C.c_int, C.c_float, C.c_float, C.c_float, f32p, f32p, f32p]
        lib.qbo_scene_generate.restype = C.c_int
        lib.qbo_camera_ray.argtypes = [C.POINTER(QboView), C.c_int, C.c_int, f32p]
        lib.qbo_camera_ray.restype = None
        lib.qbo_shade.argtypes = [f32p, f32p, f32p, f32p, C.c_float, C.c_int, f32p]
        lib.qbo_shade.restype = None
        _qbo = lib
    return _qbo


def ref() -> C.CDLL | None:
    """The reference's octree.c library, or None when it cannot be built here."""
    global _ref
    if _ref is None:
        if not os.path.exists(LIBREF):
            try:
                if build_reference() is None:
                    return None
            except RuntimeError:
                return None
        lib = C.CDLL(LIBREF)
        lib.qbref_build.argtypes = [f32p, C.c_long, C.c_float, C.c_int, i32p, C.c_long]
        lib.qbref_build.restype = C.c_long
        lib.qbref_build_paths.argtypes = [i32p, C.c_long, C.c_float, C.c_int, i32p, C.c_long]
        lib.qbref_build_paths.restype = C.c_long
        lib.qbref_remove.argtypes = [i32p, C.c_long, C.c_float, C.c_int, f32p, i32p, i32p]
        lib.qbref_remove.restype = None
        lib.qbref_trace.argtypes = [i32p, C.c_long, C.c_float, C.c_int, f32p, f32p, C.c_long, i32p, f32p]
        lib.qbref_trace.restype = None
        lib.qbref_load_flat.argtypes = [C.c_char_p] * 4 + [f32p, f32p, f32p, C.c_long, i32p, C.c_long,
                                                           C.POINTER(C.c_long)]
        lib.qbref_load_flat.restype = C.c_long
        lib.qbref_frame_quats.argtypes = [C.c_float, C.c_float, f32p, f32p]
        lib.qbref_frame_quats.restype = None
        lib.qbref_camera_dirs.argtypes = [f32p, f32p, f32p, f32p, C.c_long, f32p]
        lib.qbref_camera_dirs.restype = None
        lib.qbref_shade.argtypes = [f32p, f32p, f32p, f32p, C.c_float, C.c_int, f32p]
        lib.qbref_shade.restype = None
        _ref = lib
    return _ref


def _p(a: np.ndarray, t):
    return a.ctypes.data_as(t) if a is not None else None


class Scene:
    """Arrays of one scene kept alive for the oracle (static [+ dynamic]).
    boxes=True adds the CUDA library's leaf-box records (qbo_build_boxes), so
    the walk prunes as the library does; the default walks as the shader."""

    def __init__(self, s_nodes, s_col, s_nrm, d_nodes=None, d_col=None, d_nrm=None, boxes=False):
        c32 = lambda a, dt: None if a is None else np.ascontiguousarray(a, dtype=dt)  # noqa: E731
        self.arrays = [c32(s_nodes, np.int32), c32(s_col, np.float32), c32(s_nrm, np.float32),
                       c32(d_nodes, np.int32), c32(d_col, np.float32), c32(d_nrm, np.float32)]
        sc = QboScene()
        for t in range(2):
            nodes, col, nrm = self.arrays[3 * t], self.arrays[3 * t + 1], self.arrays[3 * t + 2]
            sc.tree[t].nodes = _p(nodes, i32p) if nodes is not None else None
            sc.tree[t].n_nodes = 0 if nodes is None else nodes.size // 12
            sc.model[t].col = _p(col, f32p) if col is not None else None
            sc.model[t].nrm = _p(nrm, f32p) if nrm is not None else None
            npts = 0
            if col is not None and nrm is not None:
                npts = min(col.size // 3, nrm.size // 3)
            sc.model[t].n_points = npts
        self.box_depth = [-1, -1]
        if boxes:
            lib = qbo()
            for t in range(2):
                nodes = self.arrays[3 * t]
                if nodes is None or nodes.size == 0:
                    continue
                n = nodes.size // 12
                rec = np.zeros(n * 16, np.uint32)
                depth = lib.qbo_build_boxes(_p(nodes, i32p), n, _p(rec, u32p))
                self.box_depth[t] = depth
                if depth >= 0:
                    self.arrays.append(rec)
                    sc.tree[t].cbox = _p(rec, u32p)
                    sc.tree[t].box_depth = depth
        self.c = sc


def view_setup(width, height, position, angle, lighta, quality, maxlevel, basesize, shoot=0, focal=0.0) -> QboView:
    v = QboView()
    pos = (C.c_float * 3)(*[float(x) for x in position])
    ang = (C.c_float * 3)(*[float(x) for x in angle])
    qbo().qbo_view_setup(width, height, pos, ang, lighta, int(quality), int(maxlevel), basesize, int(shoot), focal,
                         C.byref(v))
    return v


def trace(scene: Scene, basecube, maxlevel: int, pos, dir) -> QboHit:
    h = QboHit()
    bc = (C.c_float * 4)(*[float(x) for x in basecube])
    p = (C.c_float * 3)(*[float(x) for x in pos])
    d = (C.c_float * 3)(*[float(x) for x in dir])
    qbo().qbo_trace(C.byref(scene.c), bc, int(maxlevel), p, d, C.byref(h))
    return h


def render(scene: Scene, view: QboView, threads: int = 0, streams=("rgba", "rgba8", "flags", "leaf", "isp", "visits")):
    """Whole frame -> dict of numpy arrays (H, W, ...), row 0 at the bottom."""
    h, w = view.height_px, view.width_px
    shapes = {"rgba": ((h, w, 4), np.float32, f32p), "rgba8": ((h, w, 4), np.uint8, u8p),
              "flags": ((h, w), np.uint32, u32p), "leaf": ((h, w, 4), np.int32, i32p),
              "isp": ((h, w, 4), np.float32, f32p), "visits": ((h, w, 4), np.uint32, u32p)}
    out = {s: np.zeros(shapes[s][0], shapes[s][1]) for s in streams}
    fr = QboFrame()
    for s, a in out.items():
        setattr(fr, s, a.ctypes.data_as(shapes[s][2]))
    qbo().qbo_render(C.byref(scene.c), C.byref(view), C.byref(fr), int(threads))
    return out


def trace_rays(scene: Scene, basecube, maxlevel: int, pos: np.ndarray, dirs: np.ndarray, threads: int = 0) -> dict:
    """qbo_trace over a batch of rays on host threads -> status, leaf,
    model and visits arrays."""
    pos = np.ascontiguousarray(pos, np.float32).reshape(-1, 3)
    dirs = np.ascontiguousarray(dirs, np.float32).reshape(-1, 3)
    n = pos.shape[0]
    out = {"status": np.zeros(n, np.int32), "leaf": np.zeros((n, 2), np.int32), "model": np.zeros((n, 2), np.int32),
           "visits": np.zeros((n, 2), np.int32)}
    bc = (C.c_float * 4)(*[float(x) for x in basecube])
    qbo().qbo_trace_rays(C.byref(scene.c), bc, int(maxlevel), pos.ctypes.data_as(f32p), dirs.ctypes.data_as(f32p), n,
                         out["status"].ctypes.data_as(i32p), out["leaf"].ctypes.data_as(i32p),
                         out["model"].ctypes.data_as(i32p), out["visits"].ctypes.data_as(i32p), int(threads))
    return out


def remove_points(nodes: np.ndarray, points: np.ndarray, basesize: float = 1800.0, levels: int = 12):
    """octree_remove_point restatement for each point in order, editing
    nodes (a C-contiguous int32 (n, 12) array) in place -> (modind, octind),
    -1 where a walk met an empty link."""
    assert nodes.dtype == np.int32 and nodes.flags["C_CONTIGUOUS"]
    pts = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
    n = pts.shape[0]
    mod = np.full(n, -1, np.int32)
    oct_ = np.full(n, -1, np.int32)
    qbo().qbo_remove_points(nodes.ctypes.data_as(i32p), basesize, levels, pts.ctypes.data_as(f32p), n,
                            mod.ctypes.data_as(i32p), oct_.ctypes.data_as(i32p))
    return mod, oct_


def render_pixels(scene: Scene, view: QboView, px: np.ndarray, py: np.ndarray, threads: int = 0):
    """Selected pixels -> dict of arrays (n, ...)."""
    px = np.ascontiguousarray(px, np.int32)
    py = np.ascontiguousarray(py, np.int32)
    n = px.size
    out = {"rgba": np.zeros((n, 4), np.float32), "rgba8": np.zeros((n, 4), np.uint8), "flags": np.zeros(n, np.uint32),
           "leaf": np.zeros((n, 4), np.int32), "isp": np.zeros((n, 4), np.float32),
           "visits": np.zeros((n, 4), np.uint32)}
    fr = QboFrame(out["rgba"].ctypes.data_as(f32p), out["rgba8"].ctypes.data_as(u8p),
                  out["flags"].ctypes.data_as(u32p), out["leaf"].ctypes.data_as(i32p),
                  out["isp"].ctypes.data_as(f32p), out["visits"].ctypes.data_as(u32p))
    qbo().qbo_render_pixels(C.byref(scene.c), C.byref(view), px.ctypes.data_as(i32p), py.ctypes.data_as(i32p), n,
                            C.byref(fr), int(threads))
    return out


def build_tree(points: np.ndarray, basesize: float = 1800.0, levels: int = 12) -> np.ndarray:
    """octree_insert_point restatement over all points in order (model
    indices 0..n-1), in one C call."""
    pts = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
    cap = 1 + pts.shape[0] * levels
    nodes = np.empty(cap * 12, np.int32)
    length = qbo().qbo_build_tree(pts.ctypes.data_as(f32p), pts.shape[0], basesize, levels,
                                  nodes.ctypes.data_as(i32p), cap)
    assert length > 0
    return nodes[: length * 12].reshape(-1, 12).copy()


def scene_generate(kind: int, n_points: int, seed: int, n_boxes: int, box, n_spheres: int, sphere,
                   color_noise: float = 0.0, basesize: float = 1800.0, levels: int = 12):
    """The benchmark's seeded synthetic scene (points, normals, colours in
    octree-path order), the same bits as the library's qbc_scene_generate."""
    pts, nrm, col = (np.empty((n_points, 3), np.float32) for _ in range(3))
    rc = qbo().qbo_scene_generate(int(kind), int(levels), int(n_points), int(seed), float(basesize), int(n_boxes),
                                  float(box[0]), float(box[1]), int(n_spheres), float(sphere[0]), float(sphere[1]),
                                  float(color_noise), pts.ctypes.data_as(f32p), nrm.ctypes.data_as(f32p),
                                  col.ctypes.data_as(f32p))
    if rc != 0:
        raise ValueError(f"qbo_scene_generate failed ({rc})")
    return pts, nrm, col


def build_tree_paths(octets: np.ndarray, levels: int) -> np.ndarray:
    o = np.ascontiguousarray(octets, np.int32).reshape(-1, levels)
    cap = 1 + o.shape[0] * levels
    nodes = np.zeros(cap * 12, np.int32)
    length = C.c_int64(1)
    lib = qbo()
    for i in range(o.shape[0]):
        assert lib.qbo_insert_path(nodes.ctypes.data_as(i32p), C.byref(length), cap, levels, i,
                                   o[i].ctypes.data_as(i32p)) == 0
    return nodes[: length.value * 12].reshape(-1, 12).copy()


def point_octets(points: np.ndarray, basesize: float, levels: int) -> np.ndarray:
    pts = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
    out = np.zeros((pts.shape[0], levels), np.int32)
    lib = qbo()
    for i in range(pts.shape[0]):
        lib.qbo_point_octets(basesize, levels, pts[i].ctypes.data_as(f32p), out[i].ctypes.data_as(i32p))
    return out


def ref_build(points: np.ndarray, basesize: float, levels: int) -> np.ndarray:
    lib = ref()
    pts = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
    n = lib.qbref_build(pts.ctypes.data_as(f32p), pts.shape[0], basesize, levels, None, 0)
    out = np.zeros(n * 12, np.int32)
    lib.qbref_build(pts.ctypes.data_as(f32p), pts.shape[0], basesize, levels, out.ctypes.data_as(i32p), n)
    return out.reshape(-1, 12)


def ref_build_paths(octets: np.ndarray, basesize: float, levels: int) -> np.ndarray:
    lib = ref()
    o = np.zeros((octets.shape[0], 12), np.int32)
    o[:, :levels] = octets
    n = lib.qbref_build_paths(o.ctypes.data_as(i32p), o.shape[0], basesize, levels, None, 0)
    out = np.zeros(n * 12, np.int32)
    lib.qbref_build_paths(o.ctypes.data_as(i32p), o.shape[0], basesize, levels, out.ctypes.data_as(i32p), n)
    return out.reshape(-1, 12)


def ref_trace(nodes: np.ndarray, basesize: float, levels: int, pos: np.ndarray, dirs: np.ndarray):
    """The reference's octree_trace_line: (model index, leaf cube, w=-1 if none)."""
    lib = ref()
    nodes = np.ascontiguousarray(nodes, np.int32)
    pos = np.ascontiguousarray(pos, np.float32).reshape(-1, 3)
    dirs = np.ascontiguousarray(dirs, np.float32).reshape(-1, 3)
    n = pos.shape[0]
    model = np.zeros(n, np.int32)
    tlf = np.zeros((n, 4), np.float32)
    lib.qbref_trace(nodes.ctypes.data_as(i32p), nodes.size // 12, basesize, levels, pos.ctypes.data_as(f32p),
                    dirs.ctypes.data_as(f32p), n, model.ctypes.data_as(i32p), tlf.ctypes.data_as(f32p))
    return model, tlf


def ref_load_flat(prefix: str) -> dict:
    """The reference's model_load_flat on prefix.{pnt,col,nrm,rng}: point
    count, float3 arrays and range ints."""
    lib = ref()
    paths = [(prefix + e).encode() for e in (".pnt", ".col", ".nrm", ".rng")]
    rc = C.c_long()
    n = lib.qbref_load_flat(*paths, None, None, None, 0, None, 0, C.byref(rc))
    vtx, col, nrm = (np.zeros((n, 3), np.float32) for _ in range(3))
    rng = np.zeros(max(rc.value, 1), np.int32)
    lib.qbref_load_flat(*paths, vtx.ctypes.data_as(f32p), col.ctypes.data_as(f32p), nrm.ctypes.data_as(f32p), n,
                        rng.ctypes.data_as(i32p), rng.size, C.byref(rc))
    return {"points": vtx, "colors": col, "normals": nrm, "ranges": rng[:rc.value]}


def camera_rays(view: QboView, px, py) -> np.ndarray:
    """The oracle's camera ray per pixel: (n, 4) csv xyz and the flare test's
    cosine."""
    px = np.asarray(px, np.int32).ravel()
    py = np.asarray(py, np.int32).ravel()
    out = np.zeros((px.size, 4), np.float32)
    lib = qbo()
    for k in range(px.size):
        lib.qbo_camera_ray(C.byref(view), int(px[k]), int(py[k]), out[k].ctypes.data_as(f32p))
    return out


def ref_frame_quats(angle_x: float, angle_y: float):
    """The reference's mt_quat.c frame quaternions (qz, qx) of a camera angle."""
    qz = np.zeros(4, np.float32)
    qx = np.zeros(4, np.float32)
    ref().qbref_frame_quats(angle_x, angle_y, qz.ctypes.data_as(f32p), qx.ctypes.data_as(f32p))
    return qz, qx


def ref_camera_dirs(qz, qx, cfp, ctp) -> np.ndarray:
    """The reference's mt_quat.c rotation of screen points ctp (n, 2) - cfp."""
    qz, qx, cfp = (np.ascontiguousarray(a, np.float32) for a in (qz, qx, cfp))
    ctp = np.ascontiguousarray(ctp, np.float32).reshape(-1, 2)
    out = np.zeros((ctp.shape[0], 3), np.float32)
    ref().qbref_camera_dirs(qz.ctypes.data_as(f32p), qx.ctypes.data_as(f32p), cfp.ctypes.data_as(f32p),
                            ctp.ctypes.data_as(f32p), ctp.shape[0], out.ctypes.data_as(f32p))
    return out


def shade(isp, nrm, csv, light, sqr, shoot, col, reference: bool = False) -> np.ndarray:
    """Shading of hits (octree_fsh.c:431-449), rows of isp, nrm, csv (3),
    col (4), sqr: the oracle's restatement, or (reference=True) the same
    formula on the reference's own C vector helpers."""
    isp, nrm, csv = (np.ascontiguousarray(a, np.float32).reshape(-1, 3) for a in (isp, nrm, csv))
    out = np.ascontiguousarray(col, np.float32).reshape(-1, 4).copy()
    light = np.ascontiguousarray(light, np.float32)
    sqr = np.asarray(sqr, np.float32).ravel()
    fn = ref().qbref_shade if reference else qbo().qbo_shade
    for k in range(isp.shape[0]):
        fn(isp[k].ctypes.data_as(f32p), nrm[k].ctypes.data_as(f32p), csv[k].ctypes.data_as(f32p),
           light.ctypes.data_as(f32p), float(sqr[k]), int(shoot), out[k].ctypes.data_as(f32p))
    return out
