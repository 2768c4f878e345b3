"""Leaf-box pruning (QBC_OPT_BOX_PRUNE): the walk skips children whose
subtree's leaf box the ray misses. Every output stream but the per-pixel
visit counts must equal the unpruned walk's (and so the oracle's); with
pruning off the visit counts equal the oracle's too. Covered: the room scene,
a dynamic tree, an inexact basecube, maxlevels below and above the tree's
depth, rays, two-pass proposals, and edits after which the boxes are
rebuilt."""
import numpy as np
import pytest

from conftest import LEVELS, S
from helpers import bits, compare_frame, gpu_frame, oracle_scene, upload_scene

pytestmark = pytest.mark.gpu

STREAMS = ("rgba8", "rgba32f", "flags", "leaf", "isp", "visits")


@pytest.fixture
def ctx():
    import qubatron_gb300 as qb
    c = qb.OctreeGLC(0)
    yield c
    c.close()


def _views(sizes=((320, 200),), basesize=S, maxlevel=LEVELS, shoot=0):
    from qubatron_gb300 import view_setup
    poses = [((903.7, 421.3, 1702.9), (0.0, -0.3, 0.0), 0.0), ((500.2, 600.9, 1500.3), (-0.4, -0.45, 0.0), 1.1),
             ((1300.5, 300.2, 400.7), (2.5, -0.2, 0.0), 2.0)]
    return [view_setup(w, h, pos, ang, la, 10, maxlevel, basesize, shoot, 0.0)
            for (w, h), (pos, ang, la) in zip(list(sizes) * len(poses), poses)]


def _both(ctx, views, **kw):
    import qubatron_gb300._lib as L
    ctx.set_option(L.OPT_BOX_PRUNE, 1)
    if kw:
        on, _ = ctx.render_host_ex(views, STREAMS, **kw)
    else:
        on = ctx.render_host(views, STREAMS)
    ctx.set_option(L.OPT_BOX_PRUNE, 0)
    if kw:
        off, _ = ctx.render_host_ex(views, STREAMS, **kw)
    else:
        off = ctx.render_host(views, STREAMS)
    ctx.set_option(L.OPT_BOX_PRUNE, 1)
    return on, off


def _same_but_visits(on, off, where):
    v_on = v_off = 0
    for a, b in zip(on, off):
        for k in STREAMS:
            if k == "visits":
                assert (a[k] <= b[k]).all(), f"{where}: a pruned walk visited more nodes"
                v_on += int(a[k].astype(np.int64).sum())
                v_off += int(b[k].astype(np.int64).sum())
            else:
                assert np.array_equal(a[k].view(np.uint8), b[k].view(np.uint8)), f"{where}: {k}"
    return v_on, v_off


def test_pruning_keeps_every_pixel_room(ctx):
    from qubatron_gb300 import scenes
    s = scenes.make_scene(scenes.scaled_spec("room20m", 400_000))
    upload_scene(ctx, s.nodes, s.colors, s.normals)
    v_on, v_off = _same_but_visits(*_both(ctx, _views()), "room")
    assert v_on < 0.9 * v_off, (v_on, v_off)  # it prunes


def test_pruning_with_dynamic_tree_and_two_pass(ctx, floor50k_scene):
    from qubatron_gb300 import build_octree, scenes
    import qubatron_gb300._lib as L
    s = floor50k_scene
    ch = scenes.make_character(40_000, root=(800.0, 60.0, 1100.0))
    p, n = scenes.skin_reference(ch, scenes.pose_bones(ch, 1))
    upload_scene(ctx, s.nodes, s.colors, s.normals, build_octree(p), ch.colors, n)
    views = _views(shoot=1)
    _same_but_visits(*_both(ctx, views), "dynamic")
    _same_but_visits(*_both(ctx, views, two_pass=True), "two-pass")
    ctx.render_host_ex(views, STREAMS, two_pass=True, log=True)
    on, off = _both(ctx, views, two_pass=True, proposals=L.PROPOSE_LOGGED)
    for a, b in zip(on, off):
        for k in ("rgba8", "rgba32f", "flags", "isp"):
            assert np.array_equal(a[k].view(np.uint8), b[k].view(np.uint8)), k


def test_pruning_off_where_it_cannot_apply(ctx):
    """An inexact basecube (no reciprocal walk), a maxlevel below the tree's
    depth (boxes describe deeper leaves) and above it (nothing to hit)."""
    from qubatron_gb300 import build_octree, scenes
    bs = 1234.567
    spec = scenes.scaled_spec("room20m", 150_000)
    spec.basesize = bs
    pts, nrm, col = scenes.generate_points(spec)
    upload_scene(ctx, build_octree(pts, bs, LEVELS), col, nrm)
    _same_but_visits(*_both(ctx, _views(basesize=bs)), "inexact basecube")
    s = scenes.make_scene(scenes.scaled_spec("room20m", 150_000))
    upload_scene(ctx, s.nodes, s.colors, s.normals)
    for ml in (9, 11, 13):
        _same_but_visits(*_both(ctx, _views(maxlevel=ml)), f"maxlevel {ml}")


def test_pruning_rays_and_edits(ctx, floor50k_scene):
    """Ray queries prune too; after removals, uploads and rebuilds the boxes
    follow the tree."""
    import qubatron_gb300._lib as L
    s = floor50k_scene
    upload_scene(ctx, s.nodes, s.colors, s.normals)
    rng = np.random.default_rng(4)
    pos = rng.uniform(0, S, (4000, 3)).astype(np.float32)
    dirs = rng.normal(size=(4000, 3)).astype(np.float32)
    base = (0.0, S, S, S)
    got = {}
    for prune in (1, 0):
        ctx.set_option(L.OPT_BOX_PRUNE, prune)
        got[prune] = ctx.trace_rays(pos, dirs, base, LEVELS)
    ctx.set_option(L.OPT_BOX_PRUNE, 1)
    for k in ("status", "leaf", "model"):
        assert np.array_equal(got[1][k], got[0][k]), k
    for k in ("isp", "col", "nrm"):
        assert np.array_equal(bits(got[1][k]), bits(got[0][k])), k
    views = _views()
    ctx.render_host(views, ("rgba8",))  # boxes built
    ctx.remove_points(False, s.points[::3])  # links cut: boxes stay conservative
    _same_but_visits(*_both(ctx, views), "after removal")
    ctx.build_tree(False, s.points[::2], S, LEVELS)  # rebuilt: boxes rebuilt
    _same_but_visits(*_both(ctx, views), "after rebuild")
    upload_scene(ctx, s.nodes, s.colors, s.normals)  # uploaded again
    _same_but_visits(*_both(ctx, views), "after upload")


def test_unpruned_visits_match_oracle(ctx, oracle, floor50k_scene):
    """With pruning off the visit counts are the shader's, like every other
    stream."""
    import qubatron_gb300._lib as L
    from qubatron_gb300 import view_setup
    s = floor50k_scene
    upload_scene(ctx, s.nodes, s.colors, s.normals)
    ctx.set_option(L.OPT_BOX_PRUNE, 0)
    sc = oracle_scene(oracle, s.nodes, s.colors, s.normals)
    v = view_setup(320, 240, (903.7, 421.3, 1702.9), (0.0, -0.3, 0.0), 0.0, 10, LEVELS, S, 0, 0.0)
    ov = oracle.QboView.from_bytes(v.to_bytes())
    compare_frame(gpu_frame(ctx, v), oracle.render(sc, ov), "unpruned", visits=True)


def test_box_word_counter(ctx, floor50k_scene):
    """qbc_render_stats.box_words: the leaf-box words the walks read, counted
    on renders with a visits output and pruning on; at most one word per
    listed child (four per node visit of the static tree, eight with a
    dynamic tree as well)."""
    from qubatron_gb300 import build_octree, scenes
    import qubatron_gb300._lib as L
    s = scenes.make_scene(scenes.scaled_spec("room20m", 300_000))
    upload_scene(ctx, s.nodes, s.colors, s.normals)
    views = _views()
    ctx.set_option(L.OPT_BOX_PRUNE, 1)
    bufs, st = ctx.render_host_ex(views, ("rgba8", "visits"))
    visits = sum(int(b["visits"].astype(np.int64).sum()) for b in bufs)
    assert 0 < st["box_words"] <= 4 * visits, (st["box_words"], visits)
    assert st["queued"] == 0 and st["shadow_rays"] == 0  # a fused render
    _, st = ctx.render_host_ex(views, ("rgba8",))
    assert st["box_words"] == 0  # not instrumented
    ctx.set_option(L.OPT_BOX_PRUNE, 0)
    _, st = ctx.render_host_ex(views, ("rgba8", "visits"))
    assert st["box_words"] == 0  # no boxes
    ctx.set_option(L.OPT_BOX_PRUNE, 1)
    f = floor50k_scene
    ch = scenes.make_character(40_000, root=(800.0, 60.0, 1100.0))
    p, n = scenes.skin_reference(ch, scenes.pose_bones(ch, 1))
    upload_scene(ctx, f.nodes, f.colors, f.normals, build_octree(p), ch.colors, n)
    views = _views(shoot=1)
    bufs, st = ctx.render_host_ex(views, ("rgba8", "visits"), two_pass=True)
    visits = sum(int(b["visits"].astype(np.int64).sum()) for b in bufs)
    assert 0 < st["box_words"] <= 8 * visits, (st["box_words"], visits)
    assert st["shadow_rays"] > 0


def test_pruned_walk_matches_the_oracle_with_boxes(ctx, oracle, floor50k_scene):
    """With pruning on, every stream, the visit counts included, equals the
    oracle's walk with the restated filter (oracle/qbo_boxes.c): one tree and
    two trees, fused and two-pass frames, and ray queries."""
    import qubatron_gb300._lib as L
    from qubatron_gb300 import build_octree, scenes
    from test_gpu_parity import _ray_parity
    s = floor50k_scene
    ctx.set_option(L.OPT_BOX_PRUNE, 1)
    upload_scene(ctx, s.nodes, s.colors, s.normals)
    sc = oracle_scene(oracle, s.nodes, s.colors, s.normals, boxes=True)
    assert sc.box_depth[0] == LEVELS
    for v in _views():
        compare_frame(gpu_frame(ctx, v), oracle.render(sc, oracle.QboView.from_bytes(v.to_bytes())), "one tree",
                      visits=True)
    rng = np.random.default_rng(7)
    pos = rng.uniform(0, S, (3000, 3)).astype(np.float32)
    dirs = rng.normal(size=(3000, 3)).astype(np.float32)
    _ray_parity(ctx, oracle, sc, pos, dirs, visits=True)
    ch = scenes.make_character(40_000, root=(800.0, 60.0, 1100.0))
    p, n = scenes.skin_reference(ch, scenes.pose_bones(ch, 1))
    dn = build_octree(p)
    upload_scene(ctx, s.nodes, s.colors, s.normals, dn, ch.colors, n)
    sc = oracle_scene(oracle, s.nodes, s.colors, s.normals, dn, ch.colors, n, boxes=True)
    views = _views(shoot=1)
    ref = [oracle.render(sc, oracle.QboView.from_bytes(v.to_bytes())) for v in views]
    for v, r in zip(views, ref):
        compare_frame(gpu_frame(ctx, v), r, "two trees", visits=True)
    # the same frame split: a one-tree and a two-tree launch
    ctx.set_option(L.OPT_SPLIT_TREES, 1)
    for v, r in zip(views, ref):
        compare_frame(gpu_frame(ctx, v), r, "two trees, split", visits=True)
    ctx.set_option(L.OPT_SPLIT_TREES, 0)
    _ray_parity(ctx, oracle, sc, pos, dirs, visits=True)
    got, _ = ctx.render_host_ex(views, STREAMS, two_pass=True)
    for g, r in zip(got, ref):
        compare_frame(g.arrays, r, "two trees, two-pass", visits=True)


def test_boxes_refused_when_a_node_has_two_parents(ctx):
    """A node below two parents at different levels would get a box for one
    of them only: the library builds no boxes for such an array, also when
    the breadth-first walk appends no more nodes than the array holds."""
    import qubatron_gb300._lib as L
    nodes = np.zeros((40, 12), np.int32)  # nodes 17.. unreachable
    for o in range(8):
        nodes[0, o] = 1 + o
        nodes[1 + o, 0] = 9 + o
    col = np.ones((1, 3), np.float32)
    nrm = np.tile([0.0, 0.0, -1.0], (1, 1)).astype(np.float32)
    ctx.set_option(L.OPT_BOX_PRUNE, 1)
    views = _views(maxlevel=2)
    upload_scene(ctx, nodes, col, nrm)
    _, st = ctx.render_host_ex(views, ("rgba8", "visits"))
    assert st["box_words"] > 0  # a tree: boxes built and read
    dag = nodes.copy()
    dag[9, 0] = 2  # node 2 (level 1) also below node 9 (level 2)
    upload_scene(ctx, dag, col, nrm)
    _, st = ctx.render_host_ex(views, ("rgba8", "visits"))
    assert st["box_words"] == 0
