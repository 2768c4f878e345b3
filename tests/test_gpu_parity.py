"""Parity of libqbcuda (through its C ABI) with the oracle: every output
stream bit-exact (RGBA float bits, RGBA8, per-pixel flags, leaf node indices,
intersection point and t, node-visit counts). Tolerance: none; the traversal
and shading run the shader's FP32 operations in the shader's order on both
sides. The light flare uses acos(c) < 0.02 <=> c > cos(0.02) on both sides."""
import numpy as np
import pytest

from conftest import BASECUBE, LEVELS, S
from helpers import bits, compare_frame, gpu_frame, oracle_scene, upload_scene

pytestmark = pytest.mark.gpu


@pytest.fixture
def ctx():
    """A fresh context per test: buffers uploaded by one test (a dynamic
    tree, say) must not leak into the next."""
    import qubatron_gb300 as qb
    c = qb.OctreeGLC(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def floor1m():
    from qubatron_gb300 import scenes
    return scenes.make_scene("floor1m")


def _view_for_oracle(qbo, v):
    return qbo.QboView.from_bytes(v.to_bytes())


def test_view_setup_matches_oracle(lib, oracle):
    from qubatron_gb300 import view_setup
    for args in [(640, 480, (903.7, 421.3, 1702.9), (0.0, -0.3, 0.0), 0.0, 10, 12, 1800.0, 0, 415.69),
                 (1200, 800, (700.0, 150.0, 350.0), (0.7, 0.1, 0.0), 1.3, 10, 12, 1800.0, 1, 0.0),
                 (1200, 800, (700.0, 150.0, 350.0), (-2.0, -0.2, 0.0), 0.4, 7, 11, 1234.5, 0, 0.0)]:
        a = view_setup(*args)
        b = oracle.view_setup(*args)
        assert a.to_bytes() == b.to_bytes()


def test_floor1m_frame_bit_exact(ctx, oracle, floor1m):
    from qubatron_gb300 import scenes
    s = floor1m
    upload_scene(ctx, s.nodes, s.colors, s.normals)
    v = scenes.workload_views(scenes.WORKLOADS["floor1m_640x480"])[0]
    g = gpu_frame(ctx, v)
    r = oracle.render(oracle_scene(oracle, s.nodes, s.colors, s.normals), _view_for_oracle(oracle, v))
    stats = compare_frame(g, r, "floor1m 640x480")
    assert stats["primary_leaf"] > 10000 and stats["lit"] > 1000


def test_five_point_octtest_camera(ctx, oracle, five_point):
    """The reference's OCTTEST setup: 5 points, camera at (900, 900, 3000)
    outside the cube (qubatron.c:134-145), reference focal length."""
    from qubatron_gb300 import view_setup
    nodes = five_point["nodes"]
    col = np.ones((5, 3), np.float32)
    nrm = np.tile([0.0, 0.0, -1.0], (5, 1)).astype(np.float32)
    upload_scene(ctx, nodes, col, nrm)
    sc = oracle_scene(oracle, nodes, col, nrm)
    for pos, ang in [((900.0, 900.0, 3000.0), (0.0, 0.0, 0.0)), ((10.0, 700.0, 2500.0), (0.0, 0.1, 0.0))]:
        v = view_setup(400, 300, pos, ang, 0.0, 10, LEVELS, S, 0, 0.0)
        compare_frame(gpu_frame(ctx, v), oracle.render(sc, _view_for_oracle(oracle, v)), f"5-point {pos}")


def _ray_parity(ctx, oracle, sc_oracle, pos, dirs, basecube=BASECUBE, maxlevel=LEVELS, visits=False):
    g = ctx.trace_rays(pos, dirs, basecube, maxlevel)
    for i in range(len(pos)):
        h = oracle.trace(sc_oracle, basecube, maxlevel, pos[i], dirs[i])
        assert g["status"][i] == h.status, (i, pos[i], dirs[i])
        assert tuple(g["leaf"][i]) == tuple(h.leaf[:]), i
        assert tuple(g["model"][i]) == tuple(h.model[:]), i
        assert bits(g["isp"][i]).tolist() == bits(np.array(h.isp[:], np.float32)).tolist(), i
        assert bits(g["col"][i]).tolist() == bits(np.array(h.col[:], np.float32)).tolist(), i
        assert bits(g["nrm"][i]).tolist() == bits(np.array(h.nrm[:], np.float32)).tolist(), i
        if visits:
            assert tuple(g["visits"][i]) == tuple(h.visits[:]), i
    return g


def test_edge_rays_five_point(ctx, oracle, five_point):
    fx = five_point
    col = np.ones((5, 3), np.float32)
    nrm = np.tile([0.0, 0.0, -1.0], (5, 1)).astype(np.float32)
    upload_scene(ctx, fx["nodes"], col, nrm)
    g = _ray_parity(ctx, oracle, oracle_scene(oracle, fx["nodes"], col, nrm), fx["ray_pos"], fx["ray_dir"])
    # and against the reference's own octree_trace_line results
    hit = fx["ref_tlf"][:, 3] >= 0
    assert (g["status"][hit] == 1).all() and (g["status"][~hit] != 1).all()
    np.testing.assert_array_equal(g["model"][hit, 0], fx["ref_model"][hit])


def test_edge_rays_floor50k(ctx, oracle, floor50k, floor50k_scene):
    s = floor50k_scene
    upload_scene(ctx, s.nodes, s.colors, s.normals)
    g = _ray_parity(ctx, oracle, oracle_scene(oracle, s.nodes, s.colors, s.normals), floor50k["ray_pos"],
                    floor50k["ray_dir"])
    hit = floor50k["ref_tlf"][:, 3] >= 0
    assert (g["status"][hit] == 1).all() and (g["status"][~hit] != 1).all()
    np.testing.assert_array_equal(g["model"][hit, 0], floor50k["ref_model"][hit])


def test_dynamic_tree_frame(ctx, oracle, floor50k_scene):
    """Static + dynamic basecubes walked together (octree_fsh.c:313-317)."""
    from qubatron_gb300 import build_octree, view_setup
    s = floor50k_scene
    rng = np.random.default_rng(3)
    n = 30000
    dirs = rng.normal(size=(n, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    dpts = (np.array([800.0, 300.0, 900.0]) + 120.0 * dirs).astype(np.float32)
    dnrm = dirs.astype(np.float32)
    dcol = np.tile([0.9, 0.2, 0.1], (n, 1)).astype(np.float32)
    dnodes = build_octree(dpts, S, LEVELS)
    upload_scene(ctx, s.nodes, s.colors, s.normals, dnodes, dcol, dnrm)
    sc = oracle_scene(oracle, s.nodes, s.colors, s.normals, dnodes, dcol, dnrm)
    v = view_setup(480, 360, (820.3, 350.2, 1500.7), (0.05, -0.15, 0.0), 0.8, 10, LEVELS, S, 1, 0.0)
    stats = compare_frame(gpu_frame(ctx, v), oracle.render(sc, _view_for_oracle(oracle, v)), "dynamic")
    assert stats["primary_leaf"] > 1000


def test_house_scene_with_character(ctx, oracle):
    """The house scene (3 floors x 6 closed rooms) at 2M points with the
    bone-chain character in a ground-floor room, from the house workload's
    first poses at reduced size: every stream bit-exact."""
    from qubatron_gb300 import build_octree, scenes, view_setup
    s = scenes.make_scene(scenes.scaled_spec("house90m", 2_000_000))
    w = scenes.WORKLOADS["house90m_char10m_3840x2160x32"]
    ch = scenes.make_character(60_000, root=w.character_root)
    p, n = scenes.skin_reference(ch, scenes.pose_bones(ch, 2))
    dnodes = build_octree(p, S, LEVELS)
    upload_scene(ctx, s.nodes, s.colors, s.normals, dnodes, ch.colors, n)
    sc = oracle_scene(oracle, s.nodes, s.colors, s.normals, dnodes, ch.colors, n)
    for pos, ang in w.poses[:3]:
        v = view_setup(384, 216, pos, ang, 0.0, 10, LEVELS, S, 0, scenes.vertical_fov_focal(216))
        stats = compare_frame(gpu_frame(ctx, v), oracle.render(sc, _view_for_oracle(oracle, v)), f"house {pos}")
        assert stats["primary_leaf"] > 500


def test_inexact_basesize_uses_replay(ctx, oracle):
    """A basecube edge whose cube coordinates are not all representable:
    the cube of a level is then replayed from the root instead of undone."""
    from qubatron_gb300 import build_octree, scenes, view_setup
    bs = 1234.567
    spec = scenes.scaled_spec("floor1m", 40000)
    spec.basesize = bs
    pts, nrm, col = scenes.generate_points(spec)
    nodes = build_octree(pts, bs, LEVELS)
    upload_scene(ctx, nodes, col, nrm)
    sc = oracle_scene(oracle, nodes, col, nrm)
    for maxlevel in (LEVELS, 9):
        v = view_setup(320, 240, (601.3, 300.7, 1180.9), (0.2, -0.35, 0.0), 0.0, 10, maxlevel, bs, 0, 0.0)
        compare_frame(gpu_frame(ctx, v), oracle.render(sc, _view_for_oracle(oracle, v)), f"bs={bs} ml={maxlevel}")


@pytest.mark.parametrize("quality,maxlevel,shoot,lighta", [(10, 12, 0, 0.0), (9, 11, 1, 1.1), (7, 13, 0, 2.5),
                                                           (10, 0, 0, 0.0), (10, 4, 1, 0.3)])
def test_quality_maxlevel_variants(ctx, oracle, floor50k_scene, quality, maxlevel, shoot, lighta):
    from qubatron_gb300 import view_setup
    s = floor50k_scene
    upload_scene(ctx, s.nodes, s.colors, s.normals)
    sc = oracle_scene(oracle, s.nodes, s.colors, s.normals)
    v = view_setup(400, 300, (500.2, 600.9, 1500.3), (-0.4, -0.45, 0.0), lighta, quality, maxlevel, S, shoot, 0.0)
    compare_frame(gpu_frame(ctx, v), oracle.render(sc, _view_for_oracle(oracle, v)), f"q={quality} ml={maxlevel}")


def test_ranged_uploads_like_punch_hole(ctx, oracle):
    """modelutil_punch_hole (modelutil.c:345-580): remove points, re-insert
    elsewhere, upload single-node and colour ranges; the device copy must
    then render exactly what the host arrays describe."""
    from qubatron_gb300 import Octree, scenes, view_setup
    import qubatron_gb300 as qb
    pts, nrm, col = scenes.generate_points(scenes.scaled_spec("floor1m", 60000))
    tree = Octree(S, LEVELS)
    tree.insert_points(pts)
    nodes = tree.nodes
    upload_scene(ctx, nodes, col, nrm)
    rng = np.random.default_rng(8)
    touched = set()
    for i in rng.choice(len(pts), 400, replace=False):
        _, octind = tree.remove_point(pts[i])
        touched.add(octind)
    new = tree.nodes
    for octind in sorted(touched):
        ctx.upload_texbuffer_data(new, qb.GL_INT, new.nbytes, 16, octind * 48, (octind + 1) * 48,
                                  qb.OCTREE_GLC_BUFFER_STATIC_OCTREE)
    col2 = col.copy()
    col2[1000:5000] = [0.2, 0.9, 0.4]
    ctx.upload_texbuffer_data(col2, qb.GL_FLOAT, col2.nbytes, 12, 1000 * 12, 5000 * 12,
                              qb.OCTREE_GLC_BUFFER_STATIC_COLOR)
    # append: insert points again (new nodes at the end, array grows)
    tree.insert_points(pts[:3000] + np.float32(3.0), first_index=0)
    grown = tree.nodes
    ctx.upload_texbuffer_data(grown, qb.GL_INT, grown.nbytes, 16, new.nbytes, grown.nbytes,
                              qb.OCTREE_GLC_BUFFER_STATIC_OCTREE)
    for octind in range(0, new.shape[0]):
        if not np.array_equal(grown[octind], new[octind]):
            ctx.upload_texbuffer_data(grown, qb.GL_INT, grown.nbytes, 16, octind * 48, (octind + 1) * 48,
                                      qb.OCTREE_GLC_BUFFER_STATIC_OCTREE)
    assert ctx.tree_nodes(0) == grown.shape[0]
    sc = oracle_scene(oracle, grown, col2, nrm)
    v = view_setup(320, 240, (903.7, 421.3, 1702.9), (0.0, -0.3, 0.0), 0.0, 10, LEVELS, S, 0, 0.0)
    compare_frame(gpu_frame(ctx, v), oracle.render(sc, _view_for_oracle(oracle, v)), "ranged uploads")


def test_batched_views_match_single(ctx, oracle, floor50k_scene):
    """Views of uneven sizes in one launch give the same pixels as one by one."""
    from qubatron_gb300 import view_setup
    s = floor50k_scene
    upload_scene(ctx, s.nodes, s.colors, s.normals)
    views = [view_setup(w, h, (400.0 + 37 * k, 500.0, 1600.0 - 11 * k), (0.1 * k, -0.3, 0.0), 0.0, 10, LEVELS, S,
                        0, 0.0)
             for k, (w, h) in enumerate([(320, 240), (97, 61), (640, 480), (33, 17), (250, 250)])]
    batch = ctx.render_host(views, ("rgba8", "rgba32f", "flags", "leaf", "isp", "visits"))
    for v, fb in zip(views, batch):
        single = ctx.render_host([v], ("rgba8", "rgba32f", "flags", "leaf", "isp", "visits"))[0]
        for k in fb.arrays:
            np.testing.assert_array_equal(fb.arrays[k], single.arrays[k])


def test_reference_call_octree_glc_update(ctx, oracle, floor50k_scene):
    """octree_glc_update's own signature returns the RGBA8 target."""
    import qubatron_gb300 as qb
    s = floor50k_scene
    upload_scene(ctx, s.nodes, s.colors, s.normals)
    img = qb.octree_glc_update(ctx, 300.0, 200.0, (700.0, 150.0, 350.0), (0.5, 0.0, 0.0), 0.0, 10, LEVELS, S, 0)
    v = oracle.view_setup(300.0, 200.0, (700.0, 150.0, 350.0), (0.5, 0.0, 0.0), 0.0, 10, LEVELS, S, 0, 0.0)
    r = oracle.render(oracle_scene(oracle, s.nodes, s.colors, s.normals), v, streams=("rgba8",))
    np.testing.assert_array_equal(img, r["rgba8"])


def test_argument_errors(ctx):
    import qubatron_gb300 as qb
    from qubatron_gb300 import QbcError
    a = np.zeros((4, 12), np.int32)
    with pytest.raises(QbcError):
        ctx.upload_texbuffer_data(a, qb.GL_FLOAT, a.nbytes, 16, 0, a.nbytes, qb.OCTREE_GLC_BUFFER_STATIC_OCTREE)
    with pytest.raises(QbcError):
        ctx.upload_texbuffer_data(a, qb.GL_INT, a.nbytes, 7, 0, a.nbytes, qb.OCTREE_GLC_BUFFER_STATIC_OCTREE)
    with pytest.raises(QbcError):
        ctx.upload_texbuffer_data(a, qb.GL_INT, a.nbytes, 16, 48, 0, qb.OCTREE_GLC_BUFFER_STATIC_OCTREE)
    with pytest.raises(QbcError):
        ctx.upload_texbuffer_data(a, qb.GL_INT, a.nbytes, 16, 0, a.nbytes, 9)
    with pytest.raises(QbcError):
        qb.view_setup(640, 480, (0, 0, 0), (0, 0, 0), 0.0, 10, 18, S)


def test_out_of_range_indices_are_flagged(ctx, oracle):
    """Corrupt child and model indices read as empty and set the OOB flag,
    on both sides, instead of reading outside the arrays."""
    from qubatron_gb300 import build_octree, view_setup
    pts = np.array([[100.0, 100.0, 100.0], [1700.0, 1700.0, 100.0], [900.3, 50.0, 800.0]], np.float32)
    nodes = build_octree(pts, S, LEVELS)
    nodes[5, 3] = 999999          # a child beyond the array
    nodes[nodes[:, 8] == 2, 8] = 77  # a model index beyond the points
    col = np.ones((3, 3), np.float32)
    nrm = np.tile([0.0, 1.0, 0.0], (3, 1)).astype(np.float32)
    upload_scene(ctx, nodes, col, nrm)
    sc = oracle_scene(oracle, nodes, col, nrm)
    v = view_setup(200, 150, (900.0, 900.0, 3000.0), (0.0, 0.0, 0.0), 0.0, 10, LEVELS, S, 0, 0.0)
    compare_frame(gpu_frame(ctx, v), oracle.render(sc, _view_for_oracle(oracle, v)), "oob")


def test_camera_rays_match_mt_quat(lib, oracle, ctx):
    """The kernels' per-pixel camera ray (the function the render kernels
    call) against the rays the reference's mt_quat.c computes from the same
    frame quaternions (tests/golden/camera_quat.npz), bit for bit; the flare
    test's cosine against the oracle. The quaternions are taken from the
    fixture, so the check does not depend on the host's sinf."""
    import os

    import qubatron_gb300 as qb
    from conftest import GOLDEN
    g = dict(np.load(os.path.join(GOLDEN, "camera_quat.npz")))
    for vi in range(g["angle"].shape[0]):
        sw, sh, q, focal, x, y, z = g["cam"][vi]
        args = (float(sw), float(sh), (float(x), float(y), float(z)),
                (float(g["angle"][vi][0]), float(g["angle"][vi][1]), 0.0), 0.0, int(q), 12, S, 0, float(focal))
        v = qb.view_setup(*args)
        for k in range(4):
            v.qz[k] = float(g["qz"][vi][k])
            v.qx[k] = float(g["qx"][vi][k])
        m = g["view"] == vi
        got = ctx.camera_rays(v, g["px"][m], g["py"][m])
        np.testing.assert_array_equal(got[:, :3].view(np.uint32), g["csv"][m].view(np.uint32),
                                      err_msg=f"camera {vi}")
        ref = oracle.camera_rays(_view_for_oracle(oracle, v), g["px"][m], g["py"][m])
        np.testing.assert_array_equal(got.view(np.uint32), ref.view(np.uint32), err_msg=f"camera {vi} cosine")


def test_host_outputs_in_chunks_equal_device_outputs(lib, ctx, floor50k_scene):
    """A host-output render of more than 16M pixels is rendered in chunks of
    views whose copies to the host overlap the next chunk's render; every
    stream must equal the device-output render of the same views."""
    import torch

    import qubatron_gb300 as qb
    from qubatron_gb300 import view_setup
    s = floor50k_scene
    upload_scene(ctx, s.nodes, s.colors, s.normals)
    views = [view_setup(1920, 1080, (903.7 - 40 * k, 421.3, 1702.9), (0.1 * k - 0.2, -0.3, 0.0), 0.2 * k, 10,
                        LEVELS, S, 0, 0.0) for k in range(12)]
    host = ctx.render_host(views, ("rgba8", "flags", "leaf"))
    dev, outs = [], []
    for v in views:
        t = {"rgba8": torch.empty((v.height_px, v.width_px, 4), dtype=torch.uint8, device="cuda"),
             "flags": torch.empty((v.height_px, v.width_px), dtype=torch.int32, device="cuda"),
             "leaf": torch.empty((v.height_px, v.width_px, 4), dtype=torch.int32, device="cuda")}
        o = qb.Outputs()
        o.rgba8, o.flags, o.leaf = t["rgba8"].data_ptr(), t["flags"].data_ptr(), t["leaf"].data_ptr()
        dev.append(t)
        outs.append(o)
    ctx.render_views(views, outs, on_device=True)
    ctx.synchronize()
    hits = 0
    for h, d in zip(host, dev):
        assert np.array_equal(h["rgba8"], d["rgba8"].cpu().numpy())
        assert np.array_equal(h["flags"], d["flags"].cpu().numpy().view(np.uint32))
        assert np.array_equal(h["leaf"], d["leaf"].cpu().numpy())
        hits += int((h["flags"] & 1).sum())
    assert hits > 100_000
