"""The occluder-proposal network: tensor-core forward and backward against
the float64 CPU reference (oracle/mlp_ref.py, same bf16 rounding points;
tolerance 2 % of each layer's gradient norm, 0.5 % on the loss, 1e-2 on
outputs), training on logged plain shadow walks, and renders with its
proposals that stay identical to the plain result."""
import numpy as np
import pytest

from conftest import LEVELS, S
from helpers import bits, upload_scene

pytestmark = pytest.mark.gpu


@pytest.fixture
def ctx():
    import qubatron_gb300 as qb
    c = qb.OctreeGLC(0)
    yield c
    c.close()


def _data(m, seed):
    rng = np.random.default_rng(seed)
    x = rng.uniform(-1.0, 1.0, (m, 45)).astype(np.float32)
    kind = (rng.uniform(size=m) < 0.5).astype(np.int8)
    t = np.where(kind == 1, rng.uniform(0.05, 0.95, m), 2.0).astype(np.float32)
    return x, t, kind


def test_forward_matches_reference(ctx):
    from oracle import mlp_ref
    p = mlp_ref.random_params(3)
    ctx.proposal_set_params(p)
    np.testing.assert_array_equal(ctx.proposal_params(), p)
    x, _, _ = _data(500, 4)
    got = ctx.proposal_eval(x)
    _, _, ref = mlp_ref.loss_and_grad(p, x, np.zeros(500, np.float32), np.full(500, -1, np.int8))
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-2)


def test_gradient_matches_reference(ctx):
    from oracle import mlp_ref
    p = mlp_ref.random_params(5)
    ctx.proposal_set_params(p)
    x, t, kind = _data(700, 6)
    loss, g = ctx.proposal_gradient(x, t, kind)
    rloss, rg, _ = mlp_ref.loss_and_grad(p, x, t, kind)
    assert abs(loss - rloss) <= 5e-3 * abs(rloss)
    _, _, off = mlp_ref.layout()
    for i in range(8):
        a, b = g[off[i]:off[i + 1]], rg[off[i]:off[i + 1]]
        err = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-12)
        assert err < 2e-2, (i, err)


def _check_exact(plain, got, stats):
    proven = 0
    for p, g in zip(plain, got):
        for k in ("rgba8", "flags"):
            assert np.array_equal(p[k], g[k]), k
        for k in ("rgba32f", "isp"):
            assert np.array_equal(bits(p[k]), bits(g[k])), k
        pr = g["leaf"][..., 2] == -2
        assert np.array_equal(p["leaf"][..., :2], g["leaf"][..., :2])
        assert np.array_equal(p["leaf"][..., 2:][~pr], g["leaf"][..., 2:][~pr])
        assert (p["leaf"][..., 2][pr] >= 0).all()
        proven += int(pr.sum())
    assert proven == stats["proposals_proven"], (proven, stats)
    return proven


def test_train_then_propose(ctx):
    """Train on logged shadow walks of training poses; on held-out poses the
    network's proposals leave every output identical to the plain render
    (bar the skipped shadow leaf of pixels a proposal settled), with and
    without the occlusion gate; the gate only removes tries."""
    import qubatron_gb300._lib as L
    from qubatron_gb300 import QbcError, scenes, view_setup
    s = scenes.make_scene(scenes.scaled_spec("room20m", 400_000))
    upload_scene(ctx, s.nodes, s.colors, s.normals)
    train = [view_setup(192, 108, pos, ang, 0.0, 10, LEVELS, S, 0, 0.0) for pos, ang in scenes.spline_poses(7, 24)]
    held = [view_setup(192, 108, pos, ang, 0.0, 10, LEVELS, S, 0, 0.0) for pos, ang in scenes.spline_poses(8, 3)]
    with pytest.raises(QbcError):
        ctx.render_host_ex(held, ("rgba8",), two_pass=True, proposals=L.PROPOSE_MLP)  # no network yet
    n = 0
    for i in range(0, len(train), 8):
        n = ctx.proposal_collect(train[i:i + 8])
    assert n > 5000
    st = ctx.proposal_train(steps=400, batch=4096, lr=2e-3, seed=1)
    assert st["samples"] == n and 0 < st["occluded"] < n
    assert st["loss_last"] < 0.8 * st["loss_first"], st
    ALL = ("rgba8", "rgba32f", "flags", "leaf", "isp")
    plain = ctx.render_host(held, ALL)
    tried = {}
    for gate in (0, 500):
        ctx.set_option(L.OPT_PROPOSAL_GATE, gate)
        assert ctx.get_option(L.OPT_PROPOSAL_GATE) == gate
        for level in (5, 8):
            got, stats = ctx.render_host_ex(held, ALL, two_pass=True, proposals=L.PROPOSE_MLP, proposal_level=level)
            _check_exact(plain, got, stats)
            tried[gate, level] = stats["proposals_tried"]
    assert tried[0, 8] > 0 and tried[500, 8] <= tried[0, 8], tried
    # gate 1000: the network is not run, the frame is the plain two-pass one
    ctx.set_option(L.OPT_PROPOSAL_GATE, 1000)
    got, stats = ctx.render_host_ex(held, ALL, two_pass=True, proposals=L.PROPOSE_MLP)
    assert stats["proposals_tried"] == 0 and _check_exact(plain, got, stats) == 0
    # the context's level applies when the render leaves it 0
    ctx.set_option(L.OPT_PROPOSAL_GATE, 0)
    ctx.set_option(L.OPT_PROPOSAL_LEVEL, 5)
    got, st5 = ctx.render_host_ex(held, ALL, two_pass=True, proposals=L.PROPOSE_MLP)
    _check_exact(plain, got, st5)
    assert st5["proposals_tried"] == tried[0, 5], (st5, tried)
    # the autotuner sweeps the gate (off included), count and level, and
    # leaves a setting whose pixels are the plain ones
    import torch
    import qubatron_gb300 as qb
    frames = [torch.empty((v.height_px, v.width_px, 4), dtype=torch.uint8, device="cuda") for v in held]
    outs = []
    for f in frames:
        o = qb.Outputs()
        o.rgba8 = f.data_ptr()
        outs.append(o)
    r = ctx.autotune(held, outs, reps=1, two_pass=True, proposals=L.PROPOSE_MLP)
    assert r["proposal_gate"] in (1000, 900, 700, 500, 300, 0) and 1 <= r["proposal_count"] <= 3
    assert r["proposal_level"] in (5, 6, 7, 8) and r["candidates"] >= 20, r
    assert ctx.get_option(L.OPT_PROPOSAL_GATE) == r["proposal_gate"]
    got, stats = ctx.render_host_ex(held, ALL, two_pass=True, proposals=L.PROPOSE_MLP)
    _check_exact(plain, got, stats)
    with pytest.raises(QbcError):
        ctx.set_option(L.OPT_PROPOSAL_GATE, 1001)
    with pytest.raises(QbcError):
        ctx.set_option(L.OPT_PROPOSAL_LEVEL, 0)
    ctx.proposal_clear()
    with pytest.raises(QbcError):
        ctx.proposal_train(steps=1)
