"""The per-frame dynamic update as one call and inside a frame graph
(qbc_dynamic_update_run, qbc_graph_capture_dynamic): skinning with the bones
read from device memory, the dynamic tree rebuilt on the GPU without sorting,
allocation or host round trip, the normals taken from the skinned ones.

Every frame is checked bit for bit: skinned points and normals against host
float32 skinning in the same operation order, the dynamic tree against the
CPU producer (octree_insert_point order, numbering included), the frame
against the oracle, and a graph replay against the eager calls for the same
bones. Around later frames the device's free memory must not move."""
import numpy as np
import pytest

from conftest import LEVELS, S
from helpers import compare_frame, oracle_scene, upload_scene

pytestmark = pytest.mark.gpu


class Rig:
    """A character on the device: rest arrays, bones buffer, outputs."""

    def __init__(self, torch, ctx, n=40_000, root=(880.0, 430.0, 1220.0)):
        import qubatron_gb300 as qb
        from qubatron_gb300 import scenes
        self.ch = scenes.make_character(n, root=root)
        self.n = n
        self.rp = torch.from_numpy(self.ch.rest_points).cuda()
        self.rn = torch.from_numpy(self.ch.rest_normals).cuda()
        self.bone = torch.from_numpy(self.ch.bone).cuda()
        self.bones = torch.zeros((self.ch.joints.shape[0] - 1, 12), dtype=torch.float32, device="cuda")
        self.op = torch.empty_like(self.rp)
        self.on = torch.empty_like(self.rn)
        col = np.ascontiguousarray(self.ch.colors)
        ctx.upload_texbuffer_data(col, qb.GL_FLOAT, col.nbytes, 12, 0, col.nbytes, qb.OCTREE_GLC_BUFFER_DYNAMIC_COLOR)
        self.update = qb._lib.DynamicUpdate(self.rp.data_ptr(), self.rn.data_ptr(), self.bone.data_ptr(),
                                            self.bones.data_ptr(), self.op.data_ptr(), self.on.data_ptr(), n,
                                            self.bones.shape[0], LEVELS, S, 0)

    def pose(self, torch, frame):
        from qubatron_gb300 import scenes
        b = scenes.pose_bones(self.ch, frame)
        self.bones.copy_(torch.from_numpy(b))
        return b


@pytest.fixture
def env():
    torch = pytest.importorskip("torch")
    import qubatron_gb300 as qb
    ctx = qb.OctreeGLC(0)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    prev = torch.cuda.current_stream()
    torch.cuda.set_stream(stream)
    yield torch, ctx
    torch.cuda.synchronize()
    torch.cuda.set_stream(prev)
    ctx.close()


def _views():
    from qubatron_gb300 import view_setup
    return [view_setup(320, 240, (960.3, 700.2, 1700.7), (0.05, -0.2, 0.0), 0.4, 10, LEVELS, S, 0, 0.0),
            view_setup(97, 61, (1300.0, 520.0, 1500.0), (0.7, -0.3, 0.0), 1.1, 10, LEVELS, S, 1, 0.0)]


def _outputs(torch, views):
    import qubatron_gb300 as qb
    bufs, outs = [], []
    for v in views:
        b = {"rgba8": torch.zeros((v.height_px, v.width_px, 4), dtype=torch.uint8, device="cuda"),
             "leaf": torch.zeros((v.height_px, v.width_px, 4), dtype=torch.int32, device="cuda"),
             "flags": torch.zeros((v.height_px, v.width_px), dtype=torch.int32, device="cuda")}
        o = qb.Outputs()
        for k, t in b.items():
            setattr(o, k, t.data_ptr())
        bufs.append(b)
        outs.append(o)
    return bufs, outs


def _host(bufs):
    return [{k: t.cpu().numpy() for k, t in b.items()} for b in bufs]


def test_dynamic_update_each_frame(env, oracle, floor50k_scene):
    torch, ctx = env
    from qubatron_gb300 import Octree, scenes
    s = floor50k_scene
    upload_scene(ctx, s.nodes, s.colors, s.normals)
    rig = Rig(torch, ctx)
    views = _views()
    free = None
    for frame in range(4):
        b = rig.pose(torch, frame)
        if frame >= 2:
            free = torch.cuda.mem_get_info()[0]
        ctx.dynamic_update(rig.update)
        if frame >= 2:
            assert torch.cuda.mem_get_info()[0] == free, "the update allocated device memory"
        ctx.synchronize()
        p_ref, n_ref = scenes.skin_reference(rig.ch, b)
        np.testing.assert_array_equal(rig.op.cpu().numpy().view(np.uint32), p_ref.view(np.uint32))
        np.testing.assert_array_equal(rig.on.cpu().numpy().view(np.uint32), n_ref.view(np.uint32))
        t = Octree(S, LEVELS)
        t.insert_points(p_ref)
        np.testing.assert_array_equal(ctx.download_tree(True), t.nodes)
        assert ctx.tree_nodes(1) == t.nodes.shape[0]
        sc = oracle_scene(oracle, s.nodes, s.colors, s.normals, t.nodes, rig.ch.colors, n_ref)
        got = ctx.render_host(views, ("rgba8", "rgba32f", "flags", "leaf", "isp"))
        for v, g in zip(views, got):
            ref = oracle.render(sc, oracle.QboView.from_bytes(v.to_bytes()))
            compare_frame(g.arrays, ref, f"frame {frame}")


@pytest.mark.parametrize("kind", ["fused", "fused_split", "two_pass_random"])
def test_dynamic_graph_replays_equal_eager(env, floor50k_scene, kind):
    torch, ctx = env
    import qubatron_gb300 as qb
    s = floor50k_scene
    upload_scene(ctx, s.nodes, s.colors, s.normals)
    rig = Rig(torch, ctx)
    views = _views()
    # fused_split: the frame as a one-tree and a two-tree launch (its record
    # queue grown by the eager frame before the capture)
    ctx.set_option(qb._lib.OPT_SPLIT_TREES, 1 if kind == "fused_split" else 0)
    kw = {} if kind.startswith("fused") else {"two_pass": True, "proposals": qb._lib.PROPOSE_RANDOM, "seed": 7}
    gbufs, gouts = _outputs(torch, views)
    ebufs, eouts = _outputs(torch, views)
    rig.pose(torch, 0)
    g = ctx.graph_capture_dynamic(rig.update, views, gouts, **kw)
    try:
        free = torch.cuda.mem_get_info()[0]
        for frame in (1, 2, 3, 1):
            rig.pose(torch, frame)
            g.launch()
            ctx.synchronize()
            replay = _host(gbufs)
            assert torch.cuda.mem_get_info()[0] == free, "a replay allocated device memory"
            ctx.dynamic_update(rig.update)
            ctx.render_views_ex(views, eouts, True, **kw)
            ctx.synchronize()
            eager = _host(ebufs)
            for vi, (a, b) in enumerate(zip(replay, eager)):
                for k in a:
                    assert np.array_equal(a[k], b[k]), f"frame {frame}, view {vi}, {k}"
            assert sum(int((e["flags"] & 1).sum()) for e in eager) > 1000
    finally:
        g.close()


def test_dynamic_update_reports_bad_input(env, floor50k_scene):
    torch, ctx = env
    import qubatron_gb300 as qb
    s = floor50k_scene
    upload_scene(ctx, s.nodes, s.colors, s.normals)
    rig = Rig(torch, ctx, n=5000)
    b = rig.pose(torch, 0)
    # a bone that moves its points below 0: those points are left out
    b[1, 9:] = -5000.0
    rig.bones.copy_(torch.from_numpy(b))
    ctx.dynamic_update(rig.update)
    with pytest.raises(qb.QbcError) as e:
        ctx.synchronize()
    assert "point" in str(e.value)
    from qubatron_gb300 import Octree, scenes
    p_ref, _ = scenes.skin_reference(rig.ch, b)
    keep = (p_ref >= 0).all(axis=1)
    assert 0 < keep.sum() < rig.n
    # the tree holds the other points, numbered as if the bad ones were absent
    t = Octree(S, LEVELS)
    t.insert_points(p_ref[keep])
    got = ctx.download_tree(True)
    assert got.shape == t.nodes.shape
    np.testing.assert_array_equal(got[:, :8], t.nodes[:, :8])
    # model indices name the original points; the root's is 0 in both
    assert got[0, 8] == 0
    np.testing.assert_array_equal(got[1:, 8], np.flatnonzero(keep)[t.nodes[1:, 8]])
    ctx.synchronize()  # reported once
