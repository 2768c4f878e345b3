"""Generate the golden fixtures in tests/golden from the reference itself.

Run where the reference sources are checked out, giving that checkout:

    python tests/golden/make_golden.py REFERENCE_ROOT

(or set QB_REFERENCE_ROOT).

It compiles the reference's src/qubatron/octree.c and model.c
(oracle/build_ref.sh) and
records what that code produces:

* ``five_point.npz``   the 5-point OCTTEST scene of modelutil.c:91-129:
                       node array from octree_insert_point, and
                       octree_trace_line results for an edge-case ray suite;
* ``floor50k.npz``     a 50,000-point seeded floor scene: node count and
                       SHA-256 of the node array from octree_insert_point, node
                       array from octree_insert_path over the same octets,
                       octree_remove_point results, and octree_trace_line
                       results for random and edge-case rays;
* ``remove_edges.npz`` octree_remove_point called in order on the 5-point
                       tree for duplicates, misses and points just below 0
                       (walks the reference defines), with the node array
                       after each call sequence;
* ``camera_quat.npz``  frame quaternions and per-pixel camera rays from the
                       reference's mt_quat.c (--camera-only makes just this);
* ``shade_ref.npz``    the shading formula on the reference's own C vector
                       helpers (mt_vector_3d.c) for seeded inputs
                       (--shade-only makes just this);
* ``flat/small.{pnt,col,nrm,rng}`` + ``flat_small.npz``  a 2,000-point qmc
                       flat model (7 trailing bytes after the last point, a
                       partial int after the last range) and what the
                       reference's model_load_flat (src/qubatron/model.c)
                       reads from it.

octree_trace_line covers the static single-tree traversal; rays on which
more than 4 basecube faces pass the entry test overflow the reference's
hitp[4] array (undefined behaviour) and are left out.
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import qbo  # noqa: E402

S = 1800.0
LEVELS = 12
FIVE_POINTS = np.array([[10, 690, 10], [10, 340, 10], [10, 340, 690], [10, 10, 10], [690, 10, 690]], np.float32)


def edge_rays(points: np.ndarray, seed: int, n_aim: int = 600):
    """Rays that stress the traversal's tie rules: axis-parallel directions,
    cameras on bisecting planes, cell edges and corners, inside and outside
    the basecube, rays aimed exactly at points and at cell boundaries."""
    rng = np.random.default_rng(seed)
    cams = [
        (900.0, 900.0, 3000.0),   # OCTTEST camera (qubatron.c:136), outside the cube
        (700.0, 150.0, 350.0),    # default start (qubatron.c:580)
        (900.0, 420.0, 1700.0),   # on the level-0 x bisecting plane
        (900.0, 900.0, 900.0),    # centre: on all three level-0 planes
        (450.0, 450.0, 450.0),    # a level-1 cell centre
        (0.0, 900.0, 900.0),      # on the left face
        (1800.0, 0.0, 0.0),       # the one corner inside every half-open test
        (10.0, 690.0, 10.0),      # on a point
        (-300.0, 700.0, 900.0),   # outside, left
        (903.7, 421.3, 1702.9),   # generic inside
        (2500.0, 2500.0, 2500.0), # outside, far corner
    ]
    dirs_axis = [(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1), (1, 1, 0), (1, -1, 1),
                 (-1, -1, -1), (0, 1, 1), (1, 0, -1), (0.5, -0.25, -1.0), (0, 0, 0)]
    pos, dirs = [], []
    for c in cams:
        for d in dirs_axis:
            pos.append(c)
            dirs.append(d)
        for k in range(n_aim // len(cams)):
            tgt = points[rng.integers(0, len(points))].astype(np.float64)
            mode = k % 4
            if mode == 1:   # cell corner of the target's leaf
                w = S / 4096.0
                tgt = np.floor(tgt / w) * w
            elif mode == 2:  # slightly off the point
                tgt = tgt + rng.normal(0, 0.3, 3)
            elif mode == 3:  # a bisecting plane coordinate on one axis
                ax = rng.integers(0, 3)
                lvl = rng.integers(1, LEVELS)
                w = S / (2.0 ** lvl)
                tgt[ax] = np.round(tgt[ax] / w) * w
            pos.append(c)
            dirs.append(tuple(tgt - np.array(c)))
    return np.array(pos, np.float32), np.array(dirs, np.float32)


def random_rays(points: np.ndarray, seed: int, n: int):
    rng = np.random.default_rng(seed)
    pos = rng.uniform(-400.0, 2200.0, (n, 3)).astype(np.float32)
    tgt = points[rng.integers(0, len(points), n)] + rng.normal(0, 1.5, (n, 3)).astype(np.float32)
    return pos, (tgt - pos).astype(np.float32)


def keep_defined(scene: qbo.Scene, pos, dirs):
    """Drop rays on which more than 4 basecube faces pass (hitp[4] overflow)."""
    keep = np.array([qbo.trace(scene, (0.0, S, S, S), LEVELS, p, d).faces <= 4 for p, d in zip(pos, dirs)])
    return pos[keep], dirs[keep]


def floor_points(n: int):
    from qubatron_gb300 import scenes
    pts, nrm, col = scenes.generate_points(scenes.scaled_spec("floor1m", n))
    return pts, nrm, col


def camera_golden() -> None:
    """camera_quat.npz: the frame quaternions and per-pixel camera rays of the
    shader's ray generation (octree_fsh.c:401-413), computed with the
    reference's own C quaternion functions (src/mt_math/mt_quat.c:14-29) for
    the benchmark poses and edge angles. The render size, focus point and pixel
    centres come from the oracle's uniform derivation; the rotation is the
    reference's."""
    from qubatron_gb300 import scenes
    cams = []  # (width, height, quality, focal, position, angle)
    for name in ("room20m_1920x1080x16", "floor1m_mlp_1920x1080x16"):
        w = scenes.WORKLOADS[name]
        for pos, ang in w.poses:
            cams.append((w.width, w.height, w.quality, scenes.vertical_fov_focal(w.height), pos, ang))
    w = scenes.WORKLOADS["floor1m_char2m_mixed_x64"]
    for (sw, sh), (pos, ang) in list(zip(w.sizes, w.poses))[:16]:
        cams.append((sw, sh, w.quality, scenes.vertical_fov_focal(sh), pos, ang))
    for yaw in (0.0, 1e-7, 1.5707964, -1.5707964, 3.1415927, -3.1415927, 3.0, -2.5):
        for pitch in (0.0, -0.4, 0.15, 1.5, -1.5):
            # reference focal length; quality 3 gives a fractional render size
            cams.append((1280, 720, 10 if pitch != 0.15 else 3, 0.0, (903.7, 421.3, 1702.9), (yaw, pitch, 0.0)))
    rng = np.random.default_rng(16)
    rows = {k: [] for k in ("view", "px", "py", "ctp", "csv")}
    angles, qzs, qxs, dims = [], [], [], []
    for vi, (sw, sh, q, focal, pos, ang) in enumerate(cams):
        v = qbo.view_setup(float(sw), float(sh), pos, ang, 0.0, q, 12, S, 0, focal)
        qz, qx = qbo.ref_frame_quats(ang[0], ang[1])
        W, H = v.width_px, v.height_px
        px = np.concatenate([[0, W - 1, 0, W - 1, W // 2], rng.integers(0, W, 27)]).astype(np.int32)
        py = np.concatenate([[0, 0, H - 1, H - 1, H // 2], rng.integers(0, H, 27)]).astype(np.int32)
        # pixel centres as the oracle and the kernels form them
        ctp = np.stack([(px.astype(np.float32) + np.float32(0.5)) * np.float32(v.coord_scale[0]),
                        (py.astype(np.float32) + np.float32(0.5)) * np.float32(v.coord_scale[1])], 1)
        csv = qbo.ref_camera_dirs(qz, qx, np.array(v.cfp, np.float32), ctp)
        angles.append(ang[:2])
        qzs.append(qz)
        qxs.append(qx)
        dims.append((sw, sh, q, focal, *pos))
        rows["view"].append(np.full(px.size, vi, np.int32))
        rows["px"].append(px)
        rows["py"].append(py)
        rows["ctp"].append(ctp)
        rows["csv"].append(csv)
    np.savez_compressed(os.path.join(HERE, "camera_quat.npz"), angle=np.array(angles, np.float32),
                        qz=np.array(qzs, np.float32), qx=np.array(qxs, np.float32), cam=np.array(dims, np.float64),
                        **{k: np.concatenate(v) for k, v in rows.items()})
    print("camera_quat:", len(cams), "cameras,", sum(a.size for a in rows["px"]), "pixels")


def shade_golden() -> None:
    """shade_ref.npz: the shading of octree_fsh.c:431-449 computed with the
    reference's own C vector helpers (src/mt_math/mt_vector_3d.c) for seeded
    inputs in the ranges the renders produce, and edge cases (a normal facing
    away from the light or the camera, lit and unlit, shoot on and off)."""
    rng = np.random.default_rng(17)
    n = 2000
    isp = rng.uniform(0.0, S, (n, 3)).astype(np.float32)
    nrm = rng.normal(size=(n, 3)).astype(np.float32) * rng.uniform(0.3, 2.0, (n, 1)).astype(np.float32)
    csv = (rng.normal(size=(n, 3)) * rng.uniform(300.0, 1500.0, (n, 1))).astype(np.float32)
    col = np.concatenate([rng.uniform(0.0, 1.0, (n, 3)), np.ones((n, 1))], 1).astype(np.float32)
    sqr = np.where(rng.uniform(size=n) < 0.5, rng.uniform(0.0, 15.0, n), rng.uniform(15.0, 4e5, n)).astype(np.float32)
    sqr[:8] = [0.0, 15.0, np.nextafter(np.float32(15.0), np.float32(16.0)), 14.999999, 1e-9, 16.0, 3e5, 7.5]
    light = np.array([420.0, 200.0, 680.0], np.float32)
    nrm[8:16] = (light - isp[8:16]) * np.float32(-1.0)  # facing away from the light
    csv[16:24] = nrm[16:24] * np.float32(500.0)          # facing away from the camera
    out = {}
    for shoot in (0, 1):
        out[f"ref_shoot{shoot}"] = qbo.shade(isp, nrm, csv, light, sqr, shoot, col, reference=True)
    np.savez_compressed(os.path.join(HERE, "shade_ref.npz"), isp=isp, nrm=nrm, csv=csv, col=col, sqr=sqr,
                        light=light, **out)
    print("shade_ref:", n, "inputs")


def main(root: str, only=None) -> None:
    if qbo.build_reference(root) is None:
        raise SystemExit(f"reference sources not found under {root}")
    if only == "camera":
        camera_golden()
        return
    if only == "shade":
        shade_golden()
        return

    # ---- 5-point scene ----
    nodes5 = qbo.ref_build(FIVE_POINTS, S, LEVELS)
    sc5 = qbo.Scene(nodes5, np.ones((5, 3), np.float32), np.tile([0, 0, -1], (5, 1)).astype(np.float32))
    pos, dirs = keep_defined(sc5, *edge_rays(FIVE_POINTS, 11))
    model, tlf = qbo.ref_trace(nodes5, S, LEVELS, pos, dirs)
    np.savez_compressed(os.path.join(HERE, "five_point.npz"), points=FIVE_POINTS, nodes=nodes5, ray_pos=pos,
                        ray_dir=dirs, ref_model=model, ref_tlf=tlf)
    print("five_point:", nodes5.shape[0], "nodes,", len(pos), "rays,", int((tlf[:, 3] >= 0).sum()), "leaf hits")

    # ---- seeded floor scene ----
    pts, nrm, col = floor_points(50_000)
    nodes = qbo.ref_build(pts, S, LEVELS)
    octets = qbo.point_octets(pts, S, LEVELS)
    nodes_path = qbo.ref_build_paths(octets, S, LEVELS)
    sc = qbo.Scene(nodes, col, nrm)
    ep, ed = keep_defined(sc, *edge_rays(pts, 12))
    rp, rd = keep_defined(sc, *random_rays(pts, 13, 3000))
    pos = np.concatenate([ep, rp])
    dirs = np.concatenate([ed, rd])
    model, tlf = qbo.ref_trace(nodes, S, LEVELS, pos, dirs)
    # octree_remove_point on a copy, for 64 points
    rm = nodes.copy()
    lib = qbo.ref()
    idx = np.random.default_rng(14).choice(len(pts), 64, replace=False)
    rm_out = np.zeros((64, 2), np.int32)
    for k, i in enumerate(idx):
        m = np.zeros(1, np.int32)
        o = np.zeros(1, np.int32)
        lib.qbref_remove(rm.ctypes.data_as(qbo.i32p), rm.shape[0], S, LEVELS, pts[i].ctypes.data_as(qbo.f32p),
                         m.ctypes.data_as(qbo.i32p), o.ctypes.data_as(qbo.i32p))
        rm_out[k] = (m[0], o[0])
    np.savez_compressed(os.path.join(HERE, "floor50k.npz"), n_points=50_000,
                        nodes_sha256=np.frombuffer(hashlib.sha256(nodes.tobytes()).digest(), np.uint8),
                        n_nodes=nodes.shape[0],
                        paths_sha256=np.frombuffer(hashlib.sha256(nodes_path.tobytes()).digest(), np.uint8),
                        points_sha256=np.frombuffer(hashlib.sha256(pts.tobytes()).digest(), np.uint8),
                        remove_idx=idx.astype(np.int32), remove_out=rm_out,
                        removed_sha256=np.frombuffer(hashlib.sha256(rm.tobytes()).digest(), np.uint8),
                        ray_pos=pos, ray_dir=dirs, ref_model=model, ref_tlf=tlf)
    print("floor50k:", nodes.shape[0], "nodes,", len(pos), "rays,", int((tlf[:, 3] >= 0).sum()), "leaf hits")

    # ---- octree_remove_point edge cases on the 5-point tree ----
    rm_pts = np.array([[10, 690, 10], [10, 690, 10], [10.1, 690.1, 10.1], [10, 340, 690], [900, 900, 900],
                       [-0.1, 340, 10], [-0.2, 10, 10], [690, 10, 690], [10, 10, 10], [690.2, 10.2, 690.2],
                       [1799.9, 0.1, 0.1], [10, 340, 10]], np.float32)
    rm5 = nodes5.copy()
    rm5_out = np.full((len(rm_pts), 2), -1, np.int32)
    for k, p in enumerate(rm_pts):
        m = np.full(1, -1, np.int32)
        o = np.full(1, -1, np.int32)
        lib.qbref_remove(rm5.ctypes.data_as(qbo.i32p), rm5.shape[0], S, LEVELS, p.ctypes.data_as(qbo.f32p),
                         m.ctypes.data_as(qbo.i32p), o.ctypes.data_as(qbo.i32p))
        rm5_out[k] = (m[0], o[0])
    np.savez_compressed(os.path.join(HERE, "remove_edges.npz"), nodes=nodes5, points=rm_pts, out=rm5_out,
                        nodes_after=rm5)
    print("remove_edges:", int((rm5_out[:, 1] >= 0).sum()), "of", len(rm_pts), "removed")

    # ---- qmc flat model files, read by the reference's model_load_flat ----
    from qubatron_gb300.flatfile import write_flat
    fpts, fnrm, fcol = floor_points(2000)
    rng_ints = np.random.default_rng(15).integers(0, 2000, 3 * 40).astype(np.int32)
    os.makedirs(os.path.join(HERE, "flat"), exist_ok=True)
    prefix = os.path.join(HERE, "flat", "small")
    write_flat(prefix, fpts, fnrm, fcol, rng_ints)
    with open(prefix + ".pnt", "ab") as f:
        f.write(bytes(range(7)))  # not a whole float3: ignored by the reader
    with open(prefix + ".rng", "ab") as f:
        f.write(bytes([1, 2]))  # not a whole int: ignored
    got = qbo.ref_load_flat(prefix)
    np.savez_compressed(os.path.join(HERE, "flat_small.npz"), **got)
    print("flat_small:", got["points"].shape[0], "points,", got["ranges"].size, "range ints")

    camera_golden()
    shade_golden()


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    root = args[0] if args else qbo.REFERENCE_ROOT
    if not root:
        raise SystemExit("usage: make_golden.py REFERENCE_ROOT [--camera-only | --shade-only] (or set QB_REFERENCE_ROOT)")
    main(root, "camera" if "--camera-only" in sys.argv else ("shade" if "--shade-only" in sys.argv else None))
