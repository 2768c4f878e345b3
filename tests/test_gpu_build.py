"""GPU tree build (qbc_build_tree / qbc_build_tree_paths) against the
reference's sequential insertion: the node array must be identical, node
numbering included, to octree_insert_point / octree_insert_path run over the
same points in the same order (fixtures recorded from the reference's own
octree.c, and the library's CPU producer for other orders)."""
import hashlib

import numpy as np
import pytest

from conftest import LEVELS, S
from helpers import compare_frame, gpu_frame, oracle_scene

pytestmark = pytest.mark.gpu


@pytest.fixture
def ctx():
    import qubatron_gb300 as qb
    c = qb.OctreeGLC(0)
    yield c
    c.close()


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).digest()


def test_gpu_build_matches_reference_insert_point(ctx, floor50k, floor50k_scene):
    n = ctx.build_tree(False, floor50k_scene.points, S, LEVELS)
    assert n == int(floor50k["n_nodes"])
    nodes = ctx.download_tree(False)
    assert sha(nodes) == floor50k["nodes_sha256"].tobytes()


def test_gpu_build_matches_reference_insert_path(ctx, oracle, floor50k, floor50k_scene):
    octets = oracle.point_octets(floor50k_scene.points, S, LEVELS)
    ctx.build_tree_paths(True, octets, LEVELS)
    assert sha(ctx.download_tree(True)) == floor50k["paths_sha256"].tobytes()


def test_gpu_build_any_order_with_duplicates(ctx):
    from qubatron_gb300 import Octree, scenes
    pts, _, _ = scenes.generate_points(scenes.scaled_spec("room20m", 40000))
    rng = np.random.default_rng(21)
    pts = pts[rng.permutation(len(pts))]
    pts = np.concatenate([pts, pts[:5000], pts[100:200] + np.float32(0.01)])  # repeats and near-repeats
    t = Octree(S, LEVELS)
    t.insert_points(pts, first_index=7)
    ctx.build_tree(False, pts, S, LEVELS, first_index=7)
    np.testing.assert_array_equal(ctx.download_tree(False), t.nodes)


def test_gpu_build_edge_sizes(ctx):
    from qubatron_gb300 import Octree
    assert ctx.build_tree(False, np.zeros((0, 3), np.float32), S, LEVELS) == 1
    assert not ctx.download_tree(False).any()
    one = np.array([[10.0, 690.0, 10.0]], np.float32)
    assert ctx.build_tree(False, one, S, LEVELS) == LEVELS + 1
    t = Octree(S, LEVELS)
    t.insert_points(one)
    np.testing.assert_array_equal(ctx.download_tree(False), t.nodes)
    for levels in (1, 5, 17):
        pts = np.random.default_rng(levels).uniform(0, S, (3000, 3)).astype(np.float32)
        t = Octree(S, levels)
        t.insert_points(pts)
        ctx.build_tree(False, pts, S, levels)
        np.testing.assert_array_equal(ctx.download_tree(False), t.nodes)


def test_gpu_build_rejects_bad_input(ctx):
    from qubatron_gb300 import QbcError
    with pytest.raises(QbcError):
        ctx.build_tree(False, np.array([[1.0, -2.0, 3.0]], np.float32), S, LEVELS)
    with pytest.raises(QbcError):
        ctx.build_tree_paths(False, np.full((2, LEVELS), 8, np.int32), LEVELS)


def test_render_after_gpu_build(ctx, oracle, floor50k_scene):
    """The built tree renders exactly like the same tree uploaded."""
    from qubatron_gb300 import view_setup
    s = floor50k_scene
    ctx.upload_model(False, s.colors, s.normals)
    ctx.build_tree(False, s.points, S, LEVELS)
    v = view_setup(320, 240, (903.7, 421.3, 1702.9), (0.0, -0.3, 0.0), 0.0, 10, LEVELS, S, 0, 0.0)
    r = oracle.render(oracle_scene(oracle, s.nodes, s.colors, s.normals), oracle.QboView.from_bytes(v.to_bytes()))
    compare_frame(gpu_frame(ctx, v), r, "render after GPU build")
