"""Full-size workloads on the GPU against the oracle on sampled pixels.

The 64-view character batch (1M-point floor + 2M-point character, views of
320x240 up to 3840x2160) and the house (90M points + 10M-point character,
32 views of 3840x2160) are rendered whole on the GPU, as one two-tree launch
and as a split frame. Seeded pixels of every view are compared with the
oracle's render of the same scene, pose and view: RGBA8, flags and hit-leaf
indices bit for bit. The trees are built on the GPU and read back for the
oracle (the build equals the reference's insertion, tests/test_gpu_build.py)."""
import os
import sys

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

STREAMS = ("rgba8", "flags", "leaf")


def _parity(workload: str, per_view: int, frame: int = 3, views_per_call: int = 8):
    sys.path.insert(0, ROOT)
    import bench
    import qubatron_gb300 as qb
    import qubatron_gb300._lib as L
    from oracle import qbo
    from qubatron_gb300 import scenes
    w, scene, views, character, _ = bench.prepare(workload, host_nodes=False)
    spec = scene.spec
    p, n = scenes.skin_reference(character, scenes.pose_bones(character, frame))
    ctx = qb.OctreeGLC(0)
    try:
        # trees built on the GPU (octree_insert_point numbering, equal to the
        # reference's) and read back for the oracle
        ctx.upload_model(False, scene.colors, scene.normals)
        if scene.nodes is not None:
            ctx.upload_octree(False, scene.nodes)
            snodes = scene.nodes
        else:
            ctx.build_tree(False, scene.points, spec.basesize, spec.levels)
            snodes = ctx.download_tree(False)
        ctx.upload_model(True, character.colors, n)
        ctx.build_tree(True, p, spec.basesize, spec.levels)
        dnodes = ctx.download_tree(True)
        sc = qbo.Scene(snodes, scene.colors, scene.normals, dnodes, character.colors, n)
        rng = np.random.default_rng(11)
        samples = []
        for v in views:
            ov = qbo.QboView.from_bytes(v.to_bytes())
            px = rng.integers(0, v.width_px, per_view).astype(np.int32)
            py = rng.integers(0, v.height_px, per_view).astype(np.int32)
            samples.append((px, py, qbo.render_pixels(sc, ov, px, py, os.cpu_count() or 1)))
        checked = {}
        for split in (0, 1):
            ctx.set_option(L.OPT_SPLIT_TREES, split)
            bad = {k: 0 for k in STREAMS}
            for a in range(0, len(views), views_per_call):
                got = ctx.render_host(views[a:a + views_per_call], STREAMS)
                for g, (px, py, ref) in zip(got, samples[a:a + views_per_call]):
                    f = g.arrays
                    bad["rgba8"] += int((f["rgba8"][py, px] != ref["rgba8"]).any(axis=-1).sum())
                    bad["flags"] += int((f["flags"][py, px].view(np.uint32) != ref["flags"]).sum())
                    bad["leaf"] += int((f["leaf"][py, px] != ref["leaf"]).any(axis=-1).sum())
            ctx.synchronize()
            checked[split] = bad
    finally:
        ctx.close()
    pixels = per_view * len(views)
    for split, bad in checked.items():
        assert bad == {k: 0 for k in STREAMS}, (workload, "split" if split else "one launch", bad, pixels)
    return pixels


def test_character_batch_full_size():
    """Config 4's frame: 64 mixed views, 1024 sampled pixels each."""
    assert _parity("floor1m_char2m_mixed_x64", 1024) == 65536


def test_house_full_size():
    """Config 5's frame: the 90M-point house and its character, 32 views of
    3840x2160, 512 sampled pixels each (the views go to the GPU four at a
    time, so the host buffers stay small)."""
    assert _parity("house90m_char10m_3840x2160x32", 512, views_per_call=4) == 16384
