"""The oracle's restatement of the CUDA library's leaf-box pruning
(oracle/qbo_boxes.c, no reference counterpart): the box records are
conservative (every leaf cell below a child lies inside that child's box,
checked here from each leaf's own path), arrays that are not trees get no
boxes, and a pruned walk renders every pixel of the unpruned walk with fewer
node visits."""
import numpy as np

from conftest import LEVELS, S


def _scene(n_points=20_000):
    from oracle import qbo
    from qubatron_gb300 import scenes
    spec = scenes.scaled_spec("room20m", n_points)
    pts, nrm, col = scenes.generate_points(spec)
    return qbo.build_tree(pts, spec.basesize, spec.levels), col, nrm


def _boxes(qbo, nodes):
    nodes = np.ascontiguousarray(nodes, np.int32).reshape(-1, 12)
    n = nodes.shape[0]
    rec = np.zeros(n * 16, np.uint32)
    depth = qbo.qbo().qbo_build_boxes(nodes.ctypes.data_as(qbo.i32p), n, rec.ctypes.data_as(qbo.u32p))
    return depth, rec.reshape(n, 8, 2)


def _unpack(word):
    x, y = int(word[0]), int(word[1])
    return [(x >> s) & 0xFF for s in (0, 8, 16, 24)] + [y & 0xFF, (y >> 8) & 0xFF]


def test_records_cover_every_leaf(oracle):
    nodes, _, _ = _scene()
    nodes = nodes.reshape(-1, 12)
    depth, rec = _boxes(oracle, nodes)
    assert depth == LEVELS
    checked = 0
    # walk every root-to-leaf path; at each ancestor, the leaf's cell relative
    # to the child on the path must lie inside that child's record
    stack = [(0, 0, 0, 0, 0, [])]  # node, level, cell x, y, z (octet orientation), path
    while stack:
        node, level, cx, cy, cz, path = stack.pop()
        if level == depth:
            for (anc, lev, o, ox, oy, oz) in path:
                cells = 1 << (depth - lev - 1)
                xlo, xhi, ylo, yhi, zlo, zhi = _unpack(rec[anc, o])
                for r, lo, hi in ((cx - ox, xlo, xhi), (cy - oy, ylo, yhi), (cz - oz, zlo, zhi)):
                    assert 0 <= r < cells
                    assert lo * cells <= r * 256 and (r + 1) * 256 <= (hi + 1) * cells, (anc, lev, o)
                checked += 1
            continue
        half = 1 << (depth - level - 1)
        for o in range(8):
            c = int(nodes[node, o])
            if c <= 0:
                continue
            x = cx + (half if o & 1 else 0)
            y = cy + (half if o & 2 else 0)
            z = cz + (half if o & 4 else 0)
            stack.append((c, level + 1, x, y, z, path + [(node, level, o, x, y, z)]))
    assert checked > 10_000


def test_arrays_that_are_not_trees_get_no_boxes(oracle):
    chain = np.zeros((8, 12), np.int32)
    chain[0, 0], chain[1, 0], chain[2, 0] = 1, 2, 3  # nodes 4..7 unreachable
    assert _boxes(oracle, chain)[0] == 3
    two_parents = chain.copy()
    two_parents[0, 7] = 3  # node 3 also a child of the root: levels 1 and 3
    assert _boxes(oracle, two_parents)[0] == -1
    outside = chain.copy()
    outside[2, 5] = 99
    assert _boxes(oracle, outside)[0] == -1
    cycle = chain.copy()
    cycle[3, 0] = 1
    assert _boxes(oracle, cycle)[0] == -1


def test_pruned_oracle_walk_keeps_every_pixel(oracle):
    nodes, col, nrm = _scene()
    plain = oracle.Scene(nodes, col, nrm)
    pruned = oracle.Scene(nodes, col, nrm, boxes=True)
    assert pruned.box_depth[0] == LEVELS
    for pos, ang in (((903.7, 421.3, 1702.9), (0.0, -0.3, 0.0)), ((500.2, 600.9, 1500.3), (-0.4, -0.45, 0.0))):
        v = oracle.view_setup(160, 120, pos, ang, 1.1, 10, LEVELS, S, 0, 0.0)
        a, b = oracle.render(plain, v), oracle.render(pruned, v)
        for k in ("rgba", "rgba8", "flags", "leaf", "isp"):
            assert np.array_equal(a[k].view(np.uint8), b[k].view(np.uint8)), k
        assert (b["visits"] <= a["visits"]).all()
        assert b["visits"].sum() < 0.9 * a["visits"].sum()


def test_pruned_two_tree_walk_keeps_every_pixel(oracle):
    from qubatron_gb300 import scenes
    nodes, col, nrm = _scene()
    ch = scenes.make_character(30_000, root=(800.0, 60.0, 1100.0))
    p, n = scenes.skin_reference(ch, scenes.pose_bones(ch, 1))
    dn = oracle.build_tree(p, S, LEVELS)
    plain = oracle.Scene(nodes, col, nrm, dn, ch.colors, n)
    pruned = oracle.Scene(nodes, col, nrm, dn, ch.colors, n, boxes=True)
    assert pruned.box_depth == [LEVELS, LEVELS]
    v = oracle.view_setup(160, 120, (500.2, 600.9, 1500.3), (-0.4, -0.45, 0.0), 1.1, 10, LEVELS, S, 1, 0.0)
    a, b = oracle.render(plain, v), oracle.render(pruned, v)
    for k in ("rgba", "rgba8", "flags", "leaf", "isp"):
        assert np.array_equal(a[k].view(np.uint8), b[k].view(np.uint8)), k
    assert b["visits"].sum() < a["visits"].sum()
    assert (b["visits"] <= a["visits"]).all()
    # the root rule: a primary ray that misses the leaf boxes of the dynamic
    # root's children walks the static tree alone (no dynamic visits), though
    # the shader's walk reads dynamic nodes on its way
    skipped = (b["visits"][..., 1] == 0) & (a["visits"][..., 1] > 0)
    assert skipped.sum() > 0


def test_no_pruning_where_the_filter_does_not_apply(oracle):
    """An inexact basecube, or a maxlevel below the tree's depth: the walk
    with boxes is the shader's walk, visit counts included."""
    nodes, col, nrm = _scene(5_000)
    plain = oracle.Scene(nodes, col, nrm)
    pruned = oracle.Scene(nodes, col, nrm, boxes=True)
    for bs, ml in ((1234.567, LEVELS), (S, LEVELS - 2)):
        v = oracle.view_setup(96, 64, (903.7, 421.3, 1702.9), (0.0, -0.3, 0.0), 0.0, 10, ml, bs, 0, 0.0)
        a, b = oracle.render(plain, v), oracle.render(pruned, v)
        for k in a:
            assert np.array_equal(a[k].view(np.uint8), b[k].view(np.uint8)), (bs, ml, k)
