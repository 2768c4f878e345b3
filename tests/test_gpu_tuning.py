"""Tuning options change only the time of a frame: every warp tile shape,
grid size and service threshold renders every stream bit-identically, in
the fused kernel and in the two-pass pipeline; the autotuner leaves a valid
setting applied."""
import numpy as np
import pytest
import torch

from conftest import LEVELS, S
from helpers import upload_scene

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
    # odd sizes: partial tiles of every shape at the right and top edges
    return [view_setup(w, h, pos, ang, la, 10, LEVELS, S, 0, 0.0) for w, h, pos, ang, la in [
        (203, 117, (903.7, 421.3, 1702.9), (0.0, -0.3, 0.0), 0.0),
        (97, 61, (500.2, 600.9, 1500.3), (-0.4, -0.45, 0.0), 1.1)]]


def _render(ctx, views, two_pass):
    if two_pass:
        got, _ = ctx.render_host_ex(views, ALL, two_pass=True)
        return got
    return ctx.render_host(views, ALL)


def _same(a, b, where):
    for p, q in zip(a, b):
        for k in ALL:
            assert np.array_equal(p[k].view(np.uint8), q[k].view(np.uint8)), f"{where}: {k}"


@pytest.mark.parametrize("two_pass", [False, True])
def test_options_do_not_change_pixels(ctx, floor50k_scene, two_pass):
    import qubatron_gb300._lib as L
    s = floor50k_scene
    upload_scene(ctx, s.nodes, s.colors, s.normals)
    views = _views()
    ref = _render(ctx, views, two_pass)
    for tw in (2, 4, 16, 32, 8):
        ctx.set_option(L.OPT_TILE_WIDTH, tw)
        for bl in (2, 0):
            ctx.set_option(L.OPT_BLOCKS_PER_SM, bl)
            for sm in (1, 32, 4):
                ctx.set_option(L.OPT_SERVICE_MIN, sm)
                _same(ref, _render(ctx, views, two_pass), f"tile {tw} blocks {bl} service {sm}")


def test_autotune(ctx, floor50k_scene):
    import qubatron_gb300 as qb
    import qubatron_gb300._lib as L
    from qubatron_gb300 import QbcError
    s = floor50k_scene
    upload_scene(ctx, s.nodes, s.colors, s.normals)
    views = _views()
    ref = ctx.render_host(views, ALL)
    frames = [torch.empty((v.height_px, v.width_px, 4), dtype=torch.uint8, device="cuda") for v in views]
    outs = []
    for f in frames:
        o = qb.Outputs()
        o.rgba8 = f.data_ptr()
        outs.append(o)
    r = ctx.autotune(views, outs, reps=3)
    assert r["tile_width"] in (2, 4, 8, 16, 32) and r["blocks_per_sm"] in (0, 2, 3, 4, 5, 6, 8)
    assert 1 <= r["service_min"] <= 16 and r["candidates"] >= 16
    assert 0 < r["ms_best"] <= r["ms_initial"]
    assert ctx.get_option(L.OPT_TILE_WIDTH) == r["tile_width"]
    assert ctx.get_option(L.OPT_BLOCKS_PER_SM) == r["blocks_per_sm"]
    assert ctx.get_option(L.OPT_SERVICE_MIN) == r["service_min"]
    _same(ref, ctx.render_host(views, ALL), "after autotune")
    for opt, bad in ((L.OPT_TILE_WIDTH, 6), (L.OPT_TILE_WIDTH, 1), (L.OPT_TILE_WIDTH, 64), (L.OPT_BLOCKS_PER_SM, 33),
                     (L.OPT_SERVICE_MIN, 0)):
        with pytest.raises(QbcError):
            ctx.set_option(opt, bad)
    with pytest.raises(QbcError):
        ctx.autotune(views, outs, reps=0)


@pytest.mark.parametrize("dynamic", [False, True])
def test_plain_schedule_renders_the_same_pixels(ctx, floor50k_scene, dynamic):
    """QBC_OPT_PERSISTENT 0 (one thread per pixel, no work queue) renders
    every stream, visit counts included, exactly as the persistent kernel,
    with one tree and with two, and against the oracle."""
    import qubatron_gb300._lib as L
    from qubatron_gb300 import scenes
    from oracle import qbo
    from helpers import compare_frame
    s = floor50k_scene
    d = (None, None, None)
    if dynamic:
        ch = scenes.make_character(20_000, root=(850.0, 430.0, 1250.0))
        d = (scenes.build_octree(ch.rest_points, S, LEVELS), ch.colors, ch.rest_normals)
    upload_scene(ctx, s.nodes, s.colors, s.normals, *d)
    views = _views()
    ref = ctx.render_host(views, ALL)
    for tw in (4, 8, 32):
        ctx.set_option(L.OPT_TILE_WIDTH, tw)
        ctx.set_option(L.OPT_PERSISTENT, 0)
        got = ctx.render_host(views, ALL)
        _same(ref, got, f"plain schedule, tile {tw}")
        ctx.set_option(L.OPT_PERSISTENT, 1)
    ctx.set_option(L.OPT_BOX_PRUNE, 0)
    ctx.set_option(L.OPT_PERSISTENT, 0)
    sc = qbo.Scene(s.nodes, s.colors, s.normals, *d)
    for v, g in zip(views, ctx.render_host(views, ALL)):
        compare_frame(g.arrays, qbo.render(sc, qbo.QboView.from_bytes(v.to_bytes())), "plain schedule", visits=True)
    with pytest.raises(Exception):
        ctx.set_option(L.OPT_PERSISTENT, 2)
