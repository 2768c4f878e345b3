"""qbc_render_views_noalloc, the render entry point that allocates nothing.

It exists for callers that cannot call cudaMalloc while rendering (a frame
loop that must not stall on an allocation, a process whose device memory is
already owned by another allocator or a fixed budget). Its only scratch, the
persistent kernel's work-queue counters, sits in static device memory; the
caller passes the views and device output buffers. These tests check, through
the C ABI, that it writes exactly what qbc_render_views writes (every output
stream bit for bit, the same tolerance as the other parity tests: none), on
two calls in a row (the counters keep the previous call's values and must be
cleared each time), and that it refuses more views than its counters cover
and host output pointers.

This file is collected last so that a run stopping at the first failure has
already run every other test.
"""
import numpy as np
import pytest

from conftest import LEVELS, S
from helpers import upload_scene

pytestmark = pytest.mark.gpu

STREAMS = (("rgba8", 4, "uint8"), ("rgba32f", 4, "float32"), ("flags", 1, "int32"), ("leaf", 4, "int32"),
           ("isp", 4, "float32"), ("visits", 4, "int32"))


def _device_outputs(torch, views, fill):
    """Device buffers for every stream of every view, pre-filled with junk."""
    import qubatron_gb300 as qb
    bufs, outs = [], []
    for v in views:
        b = {}
        o = qb.Outputs()
        for name, comps, dt in STREAMS:
            shape = (v.height_px, v.width_px) if comps == 1 else (v.height_px, v.width_px, comps)
            t = torch.full(shape, fill, dtype=getattr(torch, dt), device="cuda")
            b[name] = t
            setattr(o, name, t.data_ptr())
        bufs.append(b)
        outs.append(o)
    torch.cuda.synchronize()
    return bufs, outs


def _host(bufs):
    return [{k: t.cpu().numpy() for k, t in b.items()} for b in bufs]


def _views():
    from qubatron_gb300 import view_setup
    sizes = [(320, 240), (97, 61), (640, 480), (33, 17)]
    return [view_setup(w, h, (500.0 + 41 * k, 520.0, 1600.0 - 13 * k), (0.12 * k - 0.2, -0.35, 0.0), 0.3 * k, 10,
                       LEVELS, S, k & 1, 0.0) for k, (w, h) in enumerate(sizes)]


def test_noalloc_matches_render_views_twice(floor50k_scene):
    torch = pytest.importorskip("torch")
    import qubatron_gb300 as qb
    s = floor50k_scene
    ctx = qb.OctreeGLC(0)
    try:
        upload_scene(ctx, s.nodes, s.colors, s.normals)
        views = _views()
        ref_bufs, ref_outs = _device_outputs(torch, views, 0)
        ctx.render_views(views, ref_outs, on_device=True)
        ctx.synchronize()
        ref = _host(ref_bufs)
        assert sum(int((r["flags"] & 1).sum()) for r in ref) > 1000
        for call in range(2):
            bufs, outs = _device_outputs(torch, views, 77 + call)
            ctx.render_views_noalloc(views, outs)
            ctx.synchronize()
            got = _host(bufs)
            for vi, (g, r) in enumerate(zip(got, ref)):
                for name, _, _ in STREAMS:
                    a, b = g[name], r[name]
                    if a.dtype == np.float32:
                        a, b = a.view(np.uint32), b.view(np.uint32)
                    assert np.array_equal(a, b), f"call {call}, view {vi}, stream {name}"
    finally:
        ctx.close()


def test_noalloc_rejects_too_many_views_and_host_outputs(floor50k_scene):
    torch = pytest.importorskip("torch")
    import qubatron_gb300 as qb
    from qubatron_gb300 import QbcError, view_setup
    s = floor50k_scene
    ctx = qb.OctreeGLC(0)
    try:
        upload_scene(ctx, s.nodes, s.colors, s.normals)
        v = view_setup(16, 8, (500.0, 520.0, 1600.0), (0.0, -0.3, 0.0), 0.0, 10, LEVELS, S, 0, 0.0)
        dev = torch.zeros((8, 16, 4), dtype=torch.uint8, device="cuda")
        o = qb.Outputs()
        o.rgba8 = dev.data_ptr()
        n = qb._lib.NOALLOC_MAX_VIEWS + 1
        with pytest.raises(QbcError) as e:
            ctx.render_views_noalloc([v] * n, [o] * n)
        assert e.value.code == -1 and "maximum" in str(e.value)
        host = np.zeros((8, 16, 4), np.uint8)
        h = qb.Outputs()
        h.rgba8 = host.ctypes.data
        with pytest.raises(QbcError) as e:
            ctx.render_views_noalloc([v], [h])
        assert e.value.code == -1 and "device memory" in str(e.value)
        # the maximum itself is accepted
        m = qb._lib.NOALLOC_MAX_VIEWS
        ctx.render_views_noalloc([v] * m, [o] * m)
        ctx.synchronize()
    finally:
        ctx.close()


def test_noalloc_two_trees_without_a_render_first(floor50k_scene):
    """Both trees uploaded and no allocating render since: the call takes the
    two-tree kernel, walks without leaf boxes (none were built for these
    trees) and must equal qbc_render_views with pruning off on every stream,
    visit counts included; around its later calls the device's free memory
    does not move."""
    torch = pytest.importorskip("torch")
    import qubatron_gb300 as qb
    from qubatron_gb300 import scenes
    s = floor50k_scene
    ch = scenes.make_character(30_000, root=(620.0, 460.0, 1150.0))
    d_nodes = scenes.build_octree(ch.rest_points, S, LEVELS)
    ctx = qb.OctreeGLC(0)
    try:
        upload_scene(ctx, s.nodes, s.colors, s.normals, d_nodes, ch.colors, ch.rest_normals)
        views = _views()
        got = []
        for call in range(3):
            bufs, outs = _device_outputs(torch, views, 5 + call)
            free0 = torch.cuda.mem_get_info()[0]
            ctx.render_views_noalloc(views, outs)
            ctx.synchronize()
            if call > 0:  # the first call may load the kernels' code
                assert torch.cuda.mem_get_info()[0] == free0, f"call {call} changed the device's free memory"
            got.append(_host(bufs))
        ctx.set_option(qb._lib.OPT_BOX_PRUNE, 0)
        ref_bufs, ref_outs = _device_outputs(torch, views, 0)
        ctx.render_views(views, ref_outs, on_device=True)
        ctx.synchronize()
        ref = _host(ref_bufs)
        assert sum(int(r["visits"][..., 1].sum()) for r in ref) > 0, "no view walked the dynamic tree"
        for call, g_all in enumerate(got):
            for vi, (g, r) in enumerate(zip(g_all, ref)):
                for name, _, _ in STREAMS:
                    a, b = g[name], r[name]
                    if a.dtype == np.float32:
                        a, b = a.view(np.uint32), b.view(np.uint32)
                    assert np.array_equal(a, b), f"call {call}, view {vi}, stream {name}"
    finally:
        ctx.close()
