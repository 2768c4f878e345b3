"""The two-pass render (primary pass, compacted record queue, shade pass) and
the occluder-proposal test inside it. Plain two-pass output must equal the
fused kernel on every stream; with proposals (logged first leaves of a
previous plain render, i.e. perfect proposals, or seeded random ones) every
stream must still be identical except the shadow-leaf slot of pixels a
proposal settled (-2, not computed) and their shadow visit counts."""
import numpy as np
import pytest

from conftest import LEVELS, S
from helpers import bits, upload_scene
import qubatron_gb300._lib as qb

pytestmark = pytest.mark.gpu

ALL = ("rgba8", "rgba32f", "flags", "leaf", "isp", "visits")


@pytest.fixture
def ctx():
    import qubatron_gb300 as qb
    c = qb.OctreeGLC(0)
    yield c
    c.close()


def _views():
    from qubatron_gb300 import view_setup
    return [view_setup(w, h, pos, ang, la, 10, LEVELS, S, 0, 0.0) for w, h, pos, ang, la in [
        (320, 240, (903.7, 421.3, 1702.9), (0.0, -0.3, 0.0), 0.0),
        (200, 150, (500.2, 600.9, 1500.3), (-0.4, -0.45, 0.0), 1.1),
        (240, 120, (1300.5, 300.2, 400.7), (2.5, -0.2, 0.0), 2.0)]]


def _same_except_proven(plain, got, where):
    proven = None
    for k in ALL:
        a, b = plain[k], got[k]
        if k in ("rgba32f", "isp"):
            a, b = bits(a), bits(b)
        if k == "leaf":
            proven = (b[..., 2] == -2)
            assert (b[..., 3][proven] == -2).all()
            assert np.array_equal(a[..., :2], b[..., :2]), where
            assert np.array_equal(a[..., 2:][~proven], b[..., 2:][~proven]), where
            assert (a[..., 2][proven] >= 0).all(), where  # the plain walk found a leaf there
        elif k == "visits":
            assert np.array_equal(a[..., :2], b[..., :2]), where
        else:
            assert np.array_equal(a, b), f"{where}: stream {k}"
    return int(proven.sum())


def _check_scene(ctx, views):
    plain = ctx.render_host(views, ALL)
    two, st = ctx.render_host_ex(views, ALL, two_pass=True)
    for p, t in zip(plain, two):
        for k in ALL:
            assert np.array_equal(p[k], t[k]), f"two-pass plain, stream {k}"
    assert st["queued"] >= st["shadow_rays"] > 0 and st["proposals_tried"] == 0
    shadowed = sum(int((((f := p["flags"]) >> 2) & 1).sum() - ((f >> 4) & 1).sum()) for p in plain)

    # log the plain shadow walks, then propose exactly their first leaves
    _, st_log = ctx.render_host_ex(views, ALL, two_pass=True, log=True)
    logged, st_p = ctx.render_host_ex(views, ALL, two_pass=True, proposals=qb.PROPOSE_LOGGED)
    proven = sum(_same_except_proven(p, g.arrays, "logged proposals") for p, g in zip(plain, logged))
    assert proven == st_p["proposals_proven"]
    assert shadowed > 0 and proven > 0.5 * shadowed, (proven, shadowed)
    assert st_p["shadow_rays"] == st_log["shadow_rays"] - proven

    rnd, st_r = ctx.render_host_ex(views, ALL, two_pass=True, proposals=qb.PROPOSE_RANDOM, seed=12345)
    proven_r = sum(_same_except_proven(p, g.arrays, "random proposals") for p, g in zip(plain, rnd))
    assert proven_r == st_r["proposals_proven"] and st_r["proposals_tried"] > 0
    return proven, proven_r


def test_two_pass_and_proposals_floor(ctx, floor50k_scene):
    s = floor50k_scene
    upload_scene(ctx, s.nodes, s.colors, s.normals)
    _check_scene(ctx, _views())


def test_two_pass_and_proposals_room(ctx):
    from qubatron_gb300 import scenes
    s = scenes.make_scene(scenes.scaled_spec("room20m", 400_000))
    upload_scene(ctx, s.nodes, s.colors, s.normals)
    proven, _ = _check_scene(ctx, _views())
    assert proven > 100


def test_two_pass_with_dynamic_tree_and_inexact_cube(ctx):
    from qubatron_gb300 import build_octree, scenes, view_setup
    bs = 1234.567
    spec = scenes.scaled_spec("room20m", 200_000)
    spec.basesize = bs
    pts, nrm, col = scenes.generate_points(spec)
    nodes = build_octree(pts, bs, LEVELS)
    ch = scenes.make_character(30000, root=(600.0, 300.0, 700.0))
    dnodes = build_octree(ch.rest_points, bs, LEVELS)
    upload_scene(ctx, nodes, col, nrm, dnodes, ch.colors, ch.rest_normals)
    views = [view_setup(256, 160, (640.3, 420.9, 1100.7), scenes.aim((640.3, 420.9, 1100.7), (600, 500, 700)),
                        0.7, 10, LEVELS, bs, 1, 0.0)]
    plain = ctx.render_host(views, ALL)
    two, _ = ctx.render_host_ex(views, ALL, two_pass=True)
    for k in ALL:
        assert np.array_equal(plain[0][k], two[0][k]), k
    ctx.render_host_ex(views, ALL, two_pass=True, log=True)
    logged, st = ctx.render_host_ex(views, ALL, two_pass=True, proposals=qb.PROPOSE_LOGGED)
    _same_except_proven(plain[0].arrays, logged[0].arrays, "dynamic + inexact cube")


def test_logged_proposals_need_a_logged_render(ctx, floor50k_scene):
    from qubatron_gb300 import QbcError
    s = floor50k_scene
    upload_scene(ctx, s.nodes, s.colors, s.normals)
    with pytest.raises(QbcError):
        ctx.render_host_ex(_views(), ("rgba8",), two_pass=True, proposals=qb.PROPOSE_LOGGED)
    with pytest.raises(QbcError):
        ctx.render_host_ex(_views(), ("rgba8",), two_pass=False, proposals=qb.PROPOSE_RANDOM)
