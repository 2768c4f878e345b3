"""Shared helpers for the parity tests: upload a scene through the
reference-shaped upload API and compare library outputs with the oracle."""
import numpy as np

STREAMS = ("rgba8", "rgba32f", "flags", "leaf", "isp", "visits")


def upload_scene(ctx, s_nodes, s_col, s_nrm, d_nodes=None, d_col=None, d_nrm=None):
    ctx.upload_model(False, s_col, s_nrm)
    ctx.upload_octree(False, s_nodes)
    if d_nodes is not None:
        ctx.upload_model(True, d_col, d_nrm)
        ctx.upload_octree(True, d_nodes)


def oracle_scene(qbo, s_nodes, s_col, s_nrm, d_nodes=None, d_col=None, d_nrm=None, boxes=False):
    return qbo.Scene(s_nodes, s_col, s_nrm, d_nodes, d_col, d_nrm, boxes=boxes)


def bits(a: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(a).view(np.uint32)


def compare_frame(gpu: dict, ref: dict, where: str = "", visits: bool = False) -> dict:
    """Bit-exact comparison of every stream; returns counts for reporting.
    The per-pixel visit counts match the oracle's when both walk alike: box
    pruning off (QBC_OPT_BOX_PRUNE 0) against the plain oracle, or on against
    an oracle scene with boxes; visits=True compares them too."""
    key = {"rgba32f": "rgba"}
    for s in STREAMS:
        if s == "visits" and not visits:
            continue
        g = gpu[s]
        r = ref[key.get(s, s)]
        if s in ("rgba32f", "isp"):
            g, r = bits(g), bits(r)
        bad = g != r
        if bad.ndim > 2:
            bad = bad.any(axis=-1)
        n_bad = int(bad.sum())
        if n_bad:
            idx = np.argwhere(bad)[:5]
            detail = [(tuple(i), gpu[s][tuple(i)], ref[key.get(s, s)][tuple(i)]) for i in idx]
            raise AssertionError(f"{where}: stream {s}: {n_bad} pixels differ, e.g. {detail}")
    f = ref["flags"]
    return {"pixels": int(f.size), "primary_leaf": int((f & 1).sum()), "shaded": int(((f >> 2) & 1).sum()),
            "lit": int(((f >> 4) & 1).sum()), "discard": int(((f >> 1) & 1).sum()),
            "flare": int(((f >> 5) & 1).sum())}


def gpu_frame(ctx, view) -> dict:
    fb = ctx.render_host([view], STREAMS)[0]
    return fb.arrays
