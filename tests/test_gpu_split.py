"""Split frames (QBC_OPT_SPLIT_TREES): a fused frame with two trees runs as a
one-tree launch, which walks every ray whose two-tree walk would leave the
dynamic tree alone and hands the other pixels on, and a two-tree launch,
which finishes them. Every stream, the visit counts included, must equal the
one-launch frame's (which the oracle tests pin). Covered here: the record
queue filling up, after which the two-tree launch also renders the tiles
the one-tree launch left; the option, its checks and the handed-on count."""
import numpy as np
import pytest

from conftest import LEVELS, S
from helpers import upload_scene

pytestmark = pytest.mark.gpu

STREAMS = ("rgba8", "rgba32f", "flags", "leaf", "isp", "visits")


@pytest.fixture
def ctx():
    import qubatron_gb300 as qb
    c = qb.OctreeGLC(0)
    yield c
    c.close()


def _character_scene(ctx, floor50k_scene):
    from qubatron_gb300 import build_octree, scenes
    s = floor50k_scene
    ch = scenes.make_character(40_000, root=(800.0, 60.0, 1100.0))
    p, n = scenes.skin_reference(ch, scenes.pose_bones(ch, 1))
    upload_scene(ctx, s.nodes, s.colors, s.normals, build_octree(p), ch.colors, n)
    return p


def _same(a_frames, b_frames, where):
    for i, (a, b) in enumerate(zip(a_frames, b_frames)):
        for k in STREAMS:
            assert np.array_equal(a.arrays[k].view(np.uint8), b.arrays[k].view(np.uint8)), f"{where}: view {i} {k}"


def test_split_option(ctx):
    import qubatron_gb300._lib as L
    assert ctx.get_option(L.OPT_SPLIT_TREES) == 0
    ctx.set_option(L.OPT_SPLIT_TREES, 1)
    assert ctx.get_option(L.OPT_SPLIT_TREES) == 1
    for bad in (-1, 2):
        with pytest.raises(Exception):
            ctx.set_option(L.OPT_SPLIT_TREES, bad)


def test_split_frame_with_a_full_record_queue(ctx, floor50k_scene):
    """Cameras inside the character's leaf box: every primary ray may touch
    the character, so every pixel is handed on, the record queue (a quarter
    of the frame's pixels) fills, and the one-tree launch stops taking tiles
    before the frame is done."""
    import qubatron_gb300._lib as L
    from qubatron_gb300 import view_setup
    p = _character_scene(ctx, floor50k_scene)
    centre = tuple(float(x) for x in (p.min(0) + p.max(0)) / 2)
    views = [view_setup(1920, 1080, centre, (0.3, a, 0.0), 0.5, 10, LEVELS, S, 1, 0.0) for a in (0.0, 1.6, 3.2, 4.8)]
    pixels = sum(v.width_px * v.height_px for v in views)
    ctx.set_option(L.OPT_SPLIT_TREES, 1)
    split, st = ctx.render_host_ex(views, STREAMS)
    # a full queue: many pixels handed on, fewer than all of them
    assert 1_000_000 < st["queued"] < pixels, (st["queued"], pixels)
    ctx.set_option(L.OPT_SPLIT_TREES, 0)
    one, st1 = ctx.render_host_ex(views, STREAMS)
    assert st1["queued"] == 0
    _same(split, one, "full queue")
    # every pixel was rendered (no discard left unwritten by the handover)
    assert all((f.arrays["flags"] != 0).any() for f in split)
    ctx.synchronize()  # no device error (a record overflow would be reported here)


def test_split_frame_ordinary_views(ctx, floor50k_scene):
    """Views of the whole floor with the character in sight: a part of the
    pixels handed on, the queue never full."""
    import qubatron_gb300._lib as L
    from qubatron_gb300 import view_setup
    _character_scene(ctx, floor50k_scene)
    poses = [((903.7, 421.3, 1702.9), (0.0, -0.3, 0.0), 0.0), ((500.2, 600.9, 1500.3), (-0.4, -0.45, 0.0), 1.1),
             ((1300.5, 300.2, 400.7), (2.5, -0.2, 0.0), 2.0)]
    views = [view_setup(960, 540, pos, ang, la, 10, LEVELS, S, 1, 0.0) for pos, ang, la in poses]
    ctx.set_option(L.OPT_SPLIT_TREES, 1)
    split, st = ctx.render_host_ex(views, STREAMS)
    assert 0 < st["queued"] < sum(v.width_px * v.height_px for v in views) // 4
    ctx.set_option(L.OPT_SPLIT_TREES, 0)
    one, _ = ctx.render_host_ex(views, STREAMS)
    _same(split, one, "ordinary views")
    ctx.synchronize()


def test_split_frame_mixed_depths(ctx, floor50k_scene):
    """One batch with views at the full depth and below the trees' depth
    (whose rays the box test cannot clear, so every such pixel is handed
    on): every stream equals the one-launch frame's."""
    import qubatron_gb300._lib as L
    from qubatron_gb300 import view_setup
    _character_scene(ctx, floor50k_scene)
    pose = ((500.2, 600.9, 1500.3), (-0.4, -0.45, 0.0), 1.1)
    views = [view_setup(320, 200, *pose, 10, ml, S, 1, 0.0) for ml in (LEVELS, LEVELS - 3, LEVELS)]
    ctx.set_option(L.OPT_SPLIT_TREES, 1)
    split, st = ctx.render_host_ex(views, STREAMS)
    assert st["queued"] >= 320 * 200 // 2  # at least the shallow view's hits
    ctx.set_option(L.OPT_SPLIT_TREES, 0)
    one, _ = ctx.render_host_ex(views, STREAMS)
    _same(split, one, "mixed depths")
    ctx.synchronize()
