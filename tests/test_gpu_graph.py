"""A frame captured as a CUDA graph (qbc_graph_*): replays give exactly the
eager render of the same views, an update re-targets the graph to new
uniforms, and a graph whose scene, buffers or options changed since the
capture refuses to replay until it is updated."""
import numpy as np
import pytest
import torch

from conftest import LEVELS, S
from helpers import upload_scene

pytestmark = pytest.mark.gpu


@pytest.fixture
def ctx():
    import qubatron_gb300 as qb
    c = qb.OctreeGLC(0)
    yield c
    c.close()


def _views(poses, size=(256, 144)):
    from qubatron_gb300 import view_setup
    return [view_setup(size[0], size[1], pos, ang, la, 10, LEVELS, S, 0, 0.0) for pos, ang, la in poses]


POSES_A = [((903.7, 421.3, 1702.9), (0.0, -0.3, 0.0), 0.0), ((500.2, 600.9, 1500.3), (-0.4, -0.45, 0.0), 1.1)]
POSES_B = [((1300.5, 300.2, 400.7), (2.5, -0.2, 0.0), 2.0), ((880.1, 500.3, 1600.2), (0.2, -0.5, 0.0), 0.4)]


def _device_outputs(views):
    import qubatron_gb300 as qb
    bufs, outs = [], []
    for v in views:
        rgba = torch.zeros((v.height_px, v.width_px, 4), dtype=torch.uint8, device="cuda")
        leaf = torch.zeros((v.height_px, v.width_px, 4), dtype=torch.int32, device="cuda")
        o = qb.Outputs()
        o.rgba8 = rgba.data_ptr()
        o.leaf = leaf.data_ptr()
        bufs.append((rgba, leaf))
        outs.append(o)
    return bufs, outs


def _host(bufs):
    torch.cuda.synchronize()
    return [(r.cpu().numpy().copy(), l.cpu().numpy().copy()) for r, l in bufs]


def _eager(ctx, views, **kw):
    got, _ = ctx.render_host_ex(views, ("rgba8", "leaf"), **kw)
    return [(g["rgba8"], g["leaf"]) for g in got]


def _same(a, b):
    for (ra, la), (rb, lb) in zip(a, b):
        assert np.array_equal(ra, rb) and np.array_equal(la, lb)


def test_graph_replays_and_updates_the_fused_frame(ctx, floor50k_scene):
    s = floor50k_scene
    upload_scene(ctx, s.nodes, s.colors, s.normals)
    va, vb = _views(POSES_A), _views(POSES_B)
    bufs, outs = _device_outputs(va)
    with ctx.graph_capture(va, outs) as g:
        for r, l in bufs:
            r.zero_()
            l.zero_()
        l0 = ctx.launch_count()
        g.launch()
        g.launch()
        assert ctx.launch_count() - l0 == 2  # one render kernel per replay
        _same(_host(bufs), _eager(ctx, va))
        g.update(vb)
        g.launch()
        _same(_host(bufs), _eager(ctx, vb))


def test_graph_of_the_two_pass_network_frame(ctx):
    """Primary pass, fused network inference (queue length read on the
    device), shade pass: replays equal the eager two-pass render."""
    import qubatron_gb300._lib as L
    from oracle import mlp_ref
    from qubatron_gb300 import scenes
    s = scenes.make_scene(scenes.scaled_spec("room20m", 300_000))
    upload_scene(ctx, s.nodes, s.colors, s.normals)
    p = mlp_ref.random_params(11)
    p[mlp_ref.layout()[2][7] + 3] = 3.0  # gate bias: try most proposals
    ctx.proposal_set_params(p)
    va, vb = _views(POSES_A), _views(POSES_B)
    bufs, outs = _device_outputs(va)
    kw = dict(two_pass=True, proposals=L.PROPOSE_MLP, proposal_level=6)
    with ctx.graph_capture(va, outs, **kw) as g:
        g.launch()
        _same(_host(bufs), _eager(ctx, va, **kw))
        for (ra, _), (rb, _) in zip(_eager(ctx, va, **kw), _eager(ctx, va)):
            assert np.array_equal(ra, rb)  # the proposals change no pixel
        g.update(vb)
        g.launch()
        _same(_host(bufs), _eager(ctx, vb, **kw))


def test_stale_graph_refuses_to_replay(ctx, floor50k_scene):
    import qubatron_gb300._lib as L
    from qubatron_gb300 import QbcError, scenes
    s = floor50k_scene
    upload_scene(ctx, s.nodes, s.colors, s.normals)
    va = _views(POSES_A)
    bufs, outs = _device_outputs(va)
    g = ctx.graph_capture(va, outs)
    g.launch()
    ctx.set_option(L.OPT_SERVICE_MIN, 7)  # a launch parameter of the frame
    with pytest.raises(QbcError):
        g.launch()
    g.update(va)
    g.launch()
    big = scenes.make_scene(scenes.scaled_spec("room20m", 200_000))  # larger arrays: reallocated
    upload_scene(ctx, big.nodes, big.colors, big.normals)
    with pytest.raises(QbcError):
        g.launch()
    g.update(va)
    g.launch()
    _same(_host(bufs), _eager(ctx, va))
    with pytest.raises(QbcError):
        g.update(_views(POSES_A, size=(128, 72)))  # other sizes: a new capture
    with pytest.raises(QbcError):
        g.update(va[:1])
    ctx.close()
    with pytest.raises(QbcError):
        g.launch()  # context gone: detached
    g.close()
