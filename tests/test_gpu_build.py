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


def test_load_flat_builds_and_uploads(ctx, tmp_path):
    """qbc_load_flat: the reference's static load (model_load_flat, then
    octree_insert_point per point in file order, then the uploads) with the
    build on the GPU: the node array equals the producer's (pinned to the
    reference), and the frame equals one of the same scene uploaded."""
    from qubatron_gb300 import Octree, scenes, view_setup
    from qubatron_gb300.flatfile import write_flat
    from helpers import upload_scene
    pts, nrm, col = scenes.generate_points(scenes.scaled_spec("floor1m", 60_000))
    ranges = np.arange(30, dtype=np.int32)
    prefix = str(tmp_path / "scene")
    write_flat(prefix, pts, nrm, col, ranges)
    got = ctx.load_flat(prefix)
    t = Octree(S, LEVELS)
    t.insert_points(pts)
    assert got["points"] == len(pts) and got["nodes"] == t.nodes.shape[0]
    assert np.array_equal(got["ranges"], ranges)
    np.testing.assert_array_equal(ctx.download_tree(False), t.nodes)
    v = view_setup(320, 240, (903.7, 421.3, 1702.9), (0.0, -0.3, 0.0), 0.0, 10, LEVELS, S, 0, 0.0)
    loaded = ctx.render_host([v], ("rgba8", "leaf", "isp"))[0]
    import qubatron_gb300 as qb
    with qb.OctreeGLC(0) as other:
        upload_scene(other, t.nodes, col, nrm)
        direct = other.render_host([v], ("rgba8", "leaf", "isp"))[0]
    for k in ("rgba8", "leaf", "isp"):
        assert np.array_equal(loaded[k], direct[k]), k


def test_remove_points_matches_reference(ctx, floor50k, floor50k_scene):
    """One batch of qbc_tree_remove_points equals the reference's
    octree_remove_point called in order (fixtures recorded from its own
    octree.c): reported model / parent indices and the edited node array."""
    s = floor50k_scene
    ctx.build_tree(False, s.points, S, LEVELS)
    idx = floor50k["remove_idx"]
    mod, oct_, removed = ctx.remove_points(False, s.points[idx])
    np.testing.assert_array_equal(np.stack([mod, oct_], 1), floor50k["remove_out"])
    assert removed == int((floor50k["remove_out"][:, 1] >= 0).sum())
    assert sha(ctx.download_tree(False)) == floor50k["removed_sha256"].tobytes()


def test_remove_points_edge_cases_match_reference(ctx):
    import os
    from conftest import ROOT
    d = np.load(os.path.join(ROOT, "tests", "golden", "remove_edges.npz"))
    from helpers import upload_scene
    n = d["nodes"]
    upload_scene(ctx, n, np.ones((5, 3), np.float32), np.ones((5, 3), np.float32))
    mod, oct_, removed = ctx.remove_points(False, d["points"])
    np.testing.assert_array_equal(np.stack([mod, oct_], 1), d["out"])
    np.testing.assert_array_equal(ctx.download_tree(False), d["nodes_after"])


def test_remove_points_batches_equal_sequential_calls(ctx):
    """Duplicates, misses and repeated batches against the producer's
    sequential octree_remove_point (itself pinned to the reference)."""
    from qubatron_gb300 import Octree, scenes
    pts, _, _ = scenes.generate_points(scenes.scaled_spec("room20m", 30000))
    t = Octree(S, LEVELS)
    t.insert_points(pts)
    ctx.build_tree(False, pts, S, LEVELS)
    rng = np.random.default_rng(5)
    for batch in range(3):
        pick = pts[rng.choice(len(pts), 700)]  # with repeats
        miss = rng.uniform(0, S, (50, 3)).astype(np.float32)
        b = np.concatenate([pick, miss, pick[:40]])[rng.permutation(790)]
        want = np.full((len(b), 2), -1, np.int32)
        for k, p in enumerate(b):
            want[k] = t.remove_point(p)
        mod, oct_, removed = ctx.remove_points(False, b)
        np.testing.assert_array_equal(np.stack([mod, oct_], 1), want)
        assert removed == int((want[:, 1] >= 0).sum()) > 0
        np.testing.assert_array_equal(ctx.download_tree(False), t.nodes)
