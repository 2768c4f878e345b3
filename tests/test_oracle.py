"""The oracle against the reference: fixtures recorded from the reference's
own octree.c (tests/golden/make_golden.py) and, where the reference sources
are present, the compiled reference itself."""
import hashlib

import numpy as np
import pytest

from conftest import BASECUBE, LEVELS, S


def sha(a: np.ndarray) -> bytes:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).digest()


def test_five_point_insert_matches_reference(oracle, five_point):
    nodes = oracle.build_tree(five_point["points"], S, LEVELS)
    np.testing.assert_array_equal(nodes, five_point["nodes"])


def test_seeded_insert_matches_reference(oracle, floor50k, floor50k_scene):
    pts = floor50k_scene.points
    assert sha(pts) == floor50k["points_sha256"].tobytes(), "scene generator drifted"
    nodes = oracle.build_tree(pts, S, LEVELS)
    assert nodes.shape[0] == int(floor50k["n_nodes"])
    assert sha(nodes) == floor50k["nodes_sha256"].tobytes()


def test_insert_path_matches_reference(oracle, floor50k, floor50k_scene):
    octets = oracle.point_octets(floor50k_scene.points, S, LEVELS)
    nodes = oracle.build_tree_paths(octets, LEVELS)
    assert sha(nodes) == floor50k["paths_sha256"].tobytes()


def test_remove_point_matches_reference(oracle, floor50k, floor50k_scene):
    nodes = oracle.build_tree(floor50k_scene.points, S, LEVELS).copy()
    lib = oracle.qbo()
    out = []
    for i in floor50k["remove_idx"]:
        m = np.zeros(1, np.int32)
        o = np.zeros(1, np.int32)
        lib.qbo_remove_point(nodes.ctypes.data_as(oracle.i32p), S, LEVELS,
                             floor50k_scene.points[i].ctypes.data_as(oracle.f32p), m.ctypes.data_as(oracle.i32p),
                             o.ctypes.data_as(oracle.i32p))
        out.append((m[0], o[0]))
    np.testing.assert_array_equal(np.array(out, np.int32), floor50k["remove_out"])
    assert sha(nodes) == floor50k["removed_sha256"].tobytes()


def _check_trace(oracle, scene, fx):
    """octree_trace_line returns the leaf's model index (0 also for a miss) and
    writes the leaf cube; the oracle must reach the same leaf on every ray."""
    n_hit = 0
    for p, d, m, tlf in zip(fx["ray_pos"], fx["ray_dir"], fx["ref_model"], fx["ref_tlf"]):
        h = oracle.trace(scene, BASECUBE, LEVELS, p, d)
        if tlf[3] >= 0:
            n_hit += 1
            assert h.status == oracle.LEAF, (p, d)
            assert h.model[0] == m
            np.testing.assert_array_equal(np.array(h.tlf[:], np.float32), tlf)
        else:
            assert h.status != oracle.LEAF, (p, d)
            assert m == 0
    return n_hit


def test_five_point_trace_matches_reference(oracle, five_point):
    fx = five_point
    sc = oracle.Scene(fx["nodes"], np.ones((5, 3), np.float32), np.tile([0, 0, -1], (5, 1)).astype(np.float32))
    assert _check_trace(oracle, sc, fx) > 100


def test_seeded_trace_matches_reference(oracle, floor50k, floor50k_scene):
    s = floor50k_scene
    sc = oracle.Scene(s.nodes, s.colors, s.normals)
    assert _check_trace(oracle, sc, floor50k) > 200


def test_live_reference_random_rays(oracle, floor50k_scene):
    """Fresh random rays against the compiled reference, when it is available."""
    if oracle.ref() is None:
        pytest.skip("reference sources not present: fixtures cover this")
    s = floor50k_scene
    sc = oracle.Scene(s.nodes, s.colors, s.normals)
    rng = np.random.default_rng(99)
    n = 2000
    pos = rng.uniform(0.0, 1800.0, (n, 3)).astype(np.float32)
    tgt = s.points[rng.integers(0, len(s.points), n)]
    dirs = (tgt - pos).astype(np.float32)
    model, tlf = oracle.ref_trace(s.nodes, S, LEVELS, pos, dirs)
    hits = 0
    for i in range(n):
        h = oracle.trace(sc, BASECUBE, LEVELS, pos[i], dirs[i])
        if h.faces > 4:
            continue
        if tlf[i][3] >= 0:
            hits += 1
            assert h.status == oracle.LEAF and h.model[0] == model[i]
            np.testing.assert_array_equal(np.array(h.tlf[:], np.float32), tlf[i])
        else:
            assert h.status != oracle.LEAF
    assert hits > 100


def test_two_tree_rules(oracle):
    """Dynamic-tree rules of the shader (octree_fsh.c:223-241, 313-317): a cell
    present only in the dynamic tree is entered; the dynamic colour wins only
    when its model index is > 0."""
    pts_s = np.array([[100.0, 100.0, 100.0]], np.float32)
    pts_d = np.array([[100.0, 100.0, 100.0], [500.0, 100.0, 100.0]], np.float32)
    ns = oracle.build_tree(pts_s, S, LEVELS)
    nd = oracle.build_tree(pts_d, S, LEVELS)
    col_s = np.array([[1.0, 0.0, 0.0]], np.float32)
    col_d = np.array([[0.0, 1.0, 0.0], [0.0, 0.0, 1.0]], np.float32)
    nrm = np.array([[0.0, 0.0, 1.0]] * 2, np.float32)
    sc = oracle.Scene(ns, col_s, nrm[:1], nd, col_d, nrm)
    # shared voxel: dynamic model index 0 -> static colour
    h = oracle.trace(sc, BASECUBE, LEVELS, (100.1, 100.1, 1700.0), (0.0, 0.0, -1.0))
    assert h.status == oracle.LEAF and h.model[1] == 0 and list(h.col[:3]) == [1.0, 0.0, 0.0]
    # dynamic-only voxel: static node 0 -> static colour of point 0, then dynamic index 1 overrides
    h = oracle.trace(sc, BASECUBE, LEVELS, (500.0, 100.0, 1700.0), (0.0, 0.0, -1.0))
    assert h.status == oracle.LEAF and h.leaf[0] == 0 and h.model[1] == 1 and list(h.col[:3]) == [0.0, 0.0, 1.0]


def test_discard_rules(oracle):
    sc = oracle.Scene(np.zeros((1, 12), np.int32), np.zeros((1, 3), np.float32), np.zeros((1, 3), np.float32))
    # outside, pointing away: fewer than 2 faces in front
    h = oracle.trace(sc, BASECUBE, LEVELS, (900.0, 900.0, 3000.0), (0.0, 0.0, 1.0))
    assert h.status == oracle.DISCARD
    # zero direction: no face at all
    h = oracle.trace(sc, BASECUBE, LEVELS, (900.0, 900.0, 900.0), (0.0, 0.0, 0.0))
    assert h.status == oracle.DISCARD and h.faces == 0
    # inside an empty tree: a miss, not a discard
    h = oracle.trace(sc, BASECUBE, LEVELS, (900.5, 900.5, 900.5), (0.3, 0.2, -1.0))
    assert h.status == oracle.MISS


def test_unorm8(oracle):
    lib = oracle.qbo()
    for f, u in [(0.0, 0), (-1.0, 0), (float("nan"), 0), (1.0, 255), (2.0, 255), (0.5, 128), (1.0 / 255.0, 1)]:
        assert lib.qbo_unorm8(f) == u


def test_batched_entry_points_equal_single_calls(oracle):
    """qbo_trace_rays (threads) and qbo_remove_points (in order) equal the
    single-ray and single-point calls they batch."""
    from qubatron_gb300 import scenes
    spec = scenes.scaled_spec("floor1m", 40_000)
    pts = scenes.generate_points(spec)[0]
    nodes = oracle.build_tree(pts, S, LEVELS)
    col = np.ones((pts.shape[0], 3), np.float32)
    sc = oracle.Scene(nodes, col, col)
    rng = np.random.default_rng(5)
    pos = rng.uniform(0, S, (1500, 3)).astype(np.float32)
    d = rng.normal(size=(1500, 3)).astype(np.float32)
    # a third of the rays aimed at surface points: many hits
    pos[:500] = (903.7, 421.3, 1702.9)
    d[:500] = pts[rng.choice(pts.shape[0], 500)] - pos[:500]
    bc = (0.0, S, S, S)
    out = oracle.trace_rays(sc, bc, LEVELS, pos, d, threads=4)
    assert (out["status"] == 1).sum() > 50
    for i in range(pos.shape[0]):
        h = oracle.trace(sc, bc, LEVELS, pos[i], d[i])
        assert (h.status, tuple(h.leaf[:]), tuple(h.model[:]), tuple(h.visits[:])) == (
            out["status"][i], tuple(out["leaf"][i]), tuple(out["model"][i]), tuple(out["visits"][i])), i
    a, b = nodes.copy(), nodes.copy()
    sel = np.concatenate([pts[rng.choice(pts.shape[0], 300, replace=False)], pts[:20]])  # with repeats
    m1, o1 = oracle.remove_points(a, sel, S, LEVELS)
    lib = oracle.qbo()
    for i in range(sel.shape[0]):
        mi, oi = np.full(1, -1, np.int32), np.full(1, -1, np.int32)
        lib.qbo_remove_point(b.ctypes.data_as(oracle.i32p), S, LEVELS, np.ascontiguousarray(sel[i]).ctypes.data_as(
            oracle.f32p), mi.ctypes.data_as(oracle.i32p), oi.ctypes.data_as(oracle.i32p))
        assert (m1[i], o1[i]) == (mi[0], oi[0]), i
    assert np.array_equal(a, b)
