"""Benchmark: primary+shadow Mrays/s of the octree ray-cast path on one GB300.

Workload (default): the room scene, 20,000,000 seeded points (closed room +
200 boxes + 100 spheres), octree depth 12, basecube 1800, rendered from 16
camera poses on a seeded Catmull-Rom spline at 1920x1080. One step renders the
16 views in one batch (one kernel launch): primary ray, shadow ray, shading and
light flare per pixel, exactly as the reference fragment shader
(src/qubatron/shaders/octree_fsh.c:399-464).

Rays per step = primary rays (one per pixel) + shadow rays actually cast
(pixels whose primary hit has t > 0) + flare rays, counted from the per-pixel
flags of one untimed frame.

value: device-resident inputs and outputs, CUDA events around each step on the
       launching stream, L2 flushed between steps (outside the events).
e2e:   the same views through the public C ABI with host output buffers
       (qbc_render_views, outputs_on_device = 0): device work plus the copy of
       every RGBA8 frame back to pinned host memory, wall clock per step.
cpu_baseline: the C oracle (a restatement of the shader, OpenMP over all host
       cores) on a seeded sample of the same pixels.

--impl reference times that CPU implementation alone (the reference's own
path is GLSL and cannot run without a graphics stack).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = "room20m_1920x1080x16"
L2_BYTES = 129 * 1024 * 1024
FALLBACK_HBM_GBS = 6800.0
# algorithmic bytes: a node visit reads one 32-byte child block of one tree;
# the leaf-box filter reads one 8-byte word per tested child; a leaf reads a
# 4-byte model index and a 12-byte colour and 12-byte normal; every pixel
# writes 4 bytes of RGBA8
BYTES_PER_VISIT = 32
BYTES_PER_BOX_WORD = 8
BYTES_PER_LEAF = 28
BYTES_PER_PIXEL_OUT = 4


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = os.path.join("/tmp", f"qb_clocks_{os.getpid()}.csv")

    def __enter__(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.fh,
                                         stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def scene_digest(scene) -> str:
    """SHA-256 of the scene's points, normals and colours: both arms of the
    benchmark state it, so they provably render the same scene."""
    import hashlib
    h = hashlib.sha256()
    for a in (scene.points, scene.normals, scene.colors):
        h.update(memoryview(np.ascontiguousarray(a)).cast("B"))
    return h.hexdigest()


def workload_config(w, scene, n_nodes: int, views) -> dict:
    """The `config` object of both arms' JSON lines: the workload alone,
    identical for the GPU arm and the reference arm."""
    pixels = sum(v.width_px * v.height_px for v in views)
    return {"workload": w.name, "points": int(scene.points.shape[0]), "nodes": int(n_nodes),
            "scene_sha256": scene_digest(scene),
            "resolution": f"{w.width}x{w.height}" if w.width else "mixed", "views": len(views), "pixels": pixels,
            "depth": 12, "basecube": 1800.0, "dynamic_points": int(w.character),
            "per_step": "re-skin + rebuild dynamic tree + render" if w.character else "render",
            "l2": "GPU arm: flushed between steps (2x L2 write, outside the timed events); node arrays "
                  f"{n_nodes * 36 / 1e9:.2f} GB > L2",
            "parallelism": "replicas only" if dist_env()[1] > 1 else "single GPU"}


def prepare_reference(workload_name: str):
    """The workload for the reference arm, built by the oracle alone (its
    scene generator, node producer and uniform derivation): this process maps
    no library of the GPU implementation."""
    from oracle import qbo
    from qubatron_gb300 import scenes
    w = scenes.WORKLOADS[workload_name]
    t = time.time()
    spec = scenes.SPECS[w.scene]
    pts, nrm, col = qbo.scene_generate(spec.kind, spec.n_points, spec.seed, spec.n_boxes, spec.box, spec.n_spheres,
                                       spec.sphere, spec.color_noise, spec.basesize, spec.levels)
    nodes = qbo.build_tree(pts, spec.basesize, spec.levels)
    scene = scenes.Scene(spec, pts, nrm, col, nodes)
    views = scenes.workload_views(w, view_setup=qbo.view_setup)
    character = scenes.make_character(w.character, root=w.character_root) if w.character else None
    return w, scene, views, character, time.time() - t


def mapped_repo_libraries() -> list:
    """Shared libraries of this repository mapped into this process."""
    out = set()
    root = os.path.realpath(ROOT)
    try:
        with open("/proc/self/maps") as f:
            for line in f:
                path = os.path.realpath(line.rsplit(None, 1)[-1]) if "/" in line else ""
                if path.startswith(root + os.sep) and ".so" in os.path.basename(path):
                    out.add(os.path.relpath(path, root))
    except OSError:
        return ["unknown: /proc/self/maps unreadable"]
    return sorted(out)


def prepare(workload_name: str, host_nodes: bool = True):
    """Scene, views and character of a workload. House-scale scenes skip the
    host node array unless host_nodes; the GPU builds their tree."""
    from qubatron_gb300 import scenes
    w = scenes.WORKLOADS[workload_name]
    t = time.time()
    spec = scenes.SPECS[w.scene]
    scene = scenes.make_scene(spec, nodes=host_nodes or spec.n_points < scenes.GPU_BUILD_POINTS)
    views = scenes.workload_views(w)
    character = scenes.make_character(w.character, root=w.character_root) if w.character else None
    return w, scene, views, character, time.time() - t


class CharacterFrames:
    """The dynamic basecube of a frame, on the device: the frame's bone set
    (pinned on the host for every frame, copied on the stream) is written
    into a device buffer that qbc_dynamic_update_run reads; it re-skins the
    character, rebuilds the dynamic tree and takes the skinned normals, with
    no allocation and no host round trip, so the whole frame can also be
    captured as one graph (qbc_graph_capture_dynamic)."""

    def __init__(self, ctx, ch, n_frames: int):
        import torch
        import qubatron_gb300 as qb
        from qubatron_gb300 import scenes
        self.qb, self.ctx, self.ch = qb, ctx, ch
        self.n = ch.rest_points.shape[0]
        self.n_bones = ch.joints.shape[0] - 1
        self.rp = torch.from_numpy(ch.rest_points).cuda()
        self.rn = torch.from_numpy(ch.rest_normals).cuda()
        self.bone = torch.from_numpy(ch.bone).cuda()
        self.op = torch.empty_like(self.rp)
        self.on = torch.empty_like(self.rn)
        self.bones_dev = torch.zeros((self.n_bones, 12), dtype=torch.float32, device="cuda")
        self.host = [torch.from_numpy(scenes.pose_bones(ch, f)).pin_memory() for f in range(n_frames)]
        self.h2d_bytes = self.n_bones * 12 * 4
        self.update = qb._lib.DynamicUpdate(self.rp.data_ptr(), self.rn.data_ptr(), self.bone.data_ptr(),
                                            self.bones_dev.data_ptr(), self.op.data_ptr(), self.on.data_ptr(), self.n,
                                            self.n_bones, 12, 1800.0, 0)
        col = np.ascontiguousarray(ch.colors)
        ctx.upload_texbuffer_data(col, qb.GL_FLOAT, col.nbytes, 12, 0, col.nbytes, qb.OCTREE_GLC_BUFFER_DYNAMIC_COLOR)
        torch.cuda.synchronize()

    def set_bones(self, frame: int):
        self.bones_dev.copy_(self.host[frame], non_blocking=True)

    def apply(self, frame: int):
        """Bones of `frame`, then the update, queued on the stream."""
        self.set_bones(frame)
        self.ctx.dynamic_update(self.update)


def count_rays(flags: np.ndarray) -> int:
    f = flags.astype(np.uint32)
    primary = f.size
    shadow = int(((f >> 2) & 1).sum())
    flare = int(((f >> 5) & 1).sum())
    return primary + shadow + flare


def cpu_sample(scene, views, budget_s: float, seed: int = 7, character=None, frame: int = 0, gpu_frames=None):
    """The oracle on a seeded pixel sample of the views, all host cores. With
    a character, its pose of `frame` is skinned and built on the host. With
    gpu_frames (per view: host arrays rgba8, flags, leaf of the same frame
    rendered on the GPU), every sampled pixel is also compared with it, after
    the timing."""
    from oracle import qbo
    threads = os.cpu_count() or 1
    if character is not None:
        from qubatron_gb300 import scenes
        p, n = scenes.skin_reference(character, scenes.pose_bones(character, frame))
        sc = qbo.Scene(scene.nodes, scene.colors, scene.normals, qbo.build_tree(p), character.colors, n)
    else:
        sc = qbo.Scene(scene.nodes, scene.colors, scene.normals)
    ov = [qbo.QboView.from_bytes(v.to_bytes()) for v in views]
    rng = np.random.default_rng(seed)

    kept = []  # (view, px, py, oracle outputs) for the parity check

    def run(per_view: int):
        rays, t0 = 0, time.perf_counter()
        for vi, v in enumerate(ov):
            px = rng.integers(0, v.width_px, per_view).astype(np.int32)
            py = rng.integers(0, v.height_px, per_view).astype(np.int32)
            out = qbo.render_pixels(sc, v, px, py, threads)
            rays += count_rays(out["flags"])
            if gpu_frames is not None:
                kept.append((vi, px, py, out))
        return rays, time.perf_counter() - t0

    # time-boxed: batches of seeded pixels of every view until the budget is spent
    run(64)  # warm the caches and the thread pool
    rays, dt, per_view, rounds = 0, 0.0, 2048, 0
    while dt < budget_s:
        r, t = run(per_view)
        rays += r
        dt += t
        rounds += 1
        if t < budget_s / 8:
            per_view *= 2
    res = {"value": rays / dt / 1e6, "unit": "Mrays/s", "cores": threads, "kind": "port",
           "sample": f"{rounds} rounds of seeded pixels over all {len(ov)} views of the same workload "
                     f"({rays} rays, {dt:.1f} s)",
           "seconds": dt, "rays": rays}
    if gpu_frames is not None:
        res["kept"] = kept
        # the GPU frame's row is py counted from the bottom (GL order), as the
        # oracle's pixel coordinates
        n = bad8 = badf = badl = 0
        for vi, px, py, out in kept:
            g = gpu_frames[vi]
            n += px.size
            bad8 += int((g["rgba8"][py, px] != out["rgba8"]).any(axis=-1).sum())
            badf += int((g["flags"][py, px].view(np.uint32) != out["flags"]).sum())
            badl += int((g["leaf"][py, px] != out["leaf"]).any(axis=-1).sum())
        res["parity"] = {"pixels": n, "rgba8_mismatch": bad8, "flags_mismatch": badf, "leaf_mismatch": badl}
    return res


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    w, scene, views, character, prep_s = prepare_reference(WORKLOAD)
    times, rays_total = [], 0
    res = None
    for step in range(args.warmup + args.steps):
        # per step a bounded sample: 6 s of CPU work at most, warm-up steps 2 s
        budget = min(args.cpu_seconds, 6.0 if step >= args.warmup else 2.0)
        res = cpu_sample(scene, views, budget_s=budget, seed=100 + step, character=character, frame=step)
        if step >= args.warmup:
            times.append(res["seconds"])
            rays_total += res["rays"]
    value = rays_total / sum(times) / 1e6
    libs = mapped_repo_libraries()
    stray = [x for x in libs if not x.startswith("oracle" + os.sep)]
    if stray:
        raise RuntimeError(f"reference arm mapped libraries of the GPU implementation: {stray}")
    line = {
        "impl": "reference", "metric": "primary+shadow Mrays/s", "value": value, "unit": "Mrays/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * statistics.mean(times) if times else None, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene)",
        "config": workload_config(w, scene, scene.nodes.shape[0], views),
        "cpu_baseline": {"value": value, "unit": "Mrays/s", "cores": res["cores"], "kind": res["kind"],
                         "sample": f"{args.steps} timed steps, {rays_total} rays in {sum(times):.1f} s; each step "
                                   f"a seeded pixel sample of the workload (last: {res['sample']})"},
        "e2e": {"value": value, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "libraries_mapped": libs,
        "prep_seconds": round(prep_s, 1),
        "note": "the reference's own path is a GLSL fragment shader (no graphics stack here); this is its C "
                "restatement (oracle/) on all host cores, per step a seeded pixel sample of the workload; the "
                "scene, node array and uniforms come from the oracle too, so no library of the GPU "
                "implementation is loaded",
    }
    print(json.dumps(line))
    return 0


def measure_e2e(ctx, views, rays, world, flush, steps, update=None, render=None, h2d_extra=0):
    """Same views through the public C ABI into pinned host buffers: the
    timed call includes the kernel and the copy of every frame to the host."""
    render = render or (lambda v, o, dev: ctx.render_views(v, o, on_device=dev))
    import torch
    import qubatron_gb300 as qb
    host = [torch.empty((v.height_px, v.width_px, 4), dtype=torch.uint8, pin_memory=True) for v in views]
    houts = []
    for h in host:
        o = qb.Outputs()
        o.rgba8 = h.data_ptr()
        houts.append(o)
    for _ in range(2):
        render(views, houts, False)
    e2e_t = []
    for k in range(max(3, steps)):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        if update:
            update(k)
        render(views, houts, False)
        e2e_t.append(time.perf_counter() - t0)
    from qubatron_gb300 import replicas
    rate, slowest_s = replicas.job_throughput(rays * len(e2e_t), sum(e2e_t), device="cuda")
    d2h = sum(h.numel() for h in host)
    h2d = len(views) * 132 + h2d_extra  # qbc_view uniforms (launch parameters), bone sets
    return {"value": rate / 1e6, "unit": "Mrays/s", "h2d_bytes_per_step": h2d,
            "d2h_bytes_per_step": d2h, "ms_per_step": 1000.0 * slowest_s / len(e2e_t)}


def time_steps(fn, stream, flush, warmup: int, steps: int):
    """warmup untimed calls, then steps calls each bracketed by CUDA events
    on `stream`, L2 flushed before each (outside the events); per-step ms."""
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for a, b in ev:
        flush.zero_()
        a.record(stream)
        fn()
        b.record(stream)
    torch.cuda.synchronize()
    return [a.elapsed_time(b) for a, b in ev]


PROPOSAL_WORKLOAD = "floor1m_mlp_1920x1080x16"


def proposal_comparison(args, device: int, stream, flush) -> dict:
    """The metric's own comparison on the learned-proposal workload (the floor
    scene, 16 held-out poses at 1920x1080): the occluder network is trained
    on the plain walk's logged shadow rays of 256 other poses (untimed), then
    four arms render the same frames, each tuned by qbc_autotune and replayed
    as a CUDA graph: plain fused persistent, plain two-pass persistent, the
    two-pass frame with network proposals, and the plain one-thread-per-pixel
    schedule. Every arm's pixels are checked against the oracle on a seeded
    sample."""
    import torch
    import qubatron_gb300 as qb
    from qubatron_gb300 import scenes
    w = scenes.WORKLOADS[PROPOSAL_WORKLOAD]
    scene = scenes.make_scene(w.scene)
    views = scenes.workload_views(w)
    ctx = qb.OctreeGLC(device)
    ctx.set_stream(stream.cuda_stream)
    ctx.upload_model(False, scene.colors, scene.normals)
    ctx.upload_octree(False, scene.nodes)
    lib = qb._lib
    out = {"workload": w.name, "points": int(scene.points.shape[0]), "nodes": int(scene.nodes.shape[0]),
           "views": len(views), "resolution": f"{w.width}x{w.height}"}
    try:
        tv = scenes.train_views(w)
        t0 = time.time()
        samples = 0
        for i in range(0, len(tv), 32):
            samples = ctx.proposal_collect(tv[i:i + 32])
        collect_s = time.time() - t0
        t0 = time.time()
        st = ctx.proposal_train(steps=args.train_steps, batch=8192, lr=2e-3, seed=1)
        torch.cuda.synchronize()
        out["training"] = {"poses": len(tv), "pose_size": "%dx%d" % w.train_size, "samples": samples,
                           "occluded": st["occluded"], "steps": args.train_steps, "batch": 8192,
                           "loss_first": st["loss_first"], "loss_last": st["loss_last"],
                           "collect_s": round(collect_s, 2), "train_s": round(time.time() - t0, 2)}
        ctx.set_option(lib.OPT_PROPOSAL_GATE, args.proposal_gate)
        ctx.set_option(lib.OPT_PROPOSAL_COUNT, args.proposal_count)
        out["proposal_options"] = {"gate_per_mille": args.proposal_gate, "count": args.proposal_count,
                                   "level": args.proposal_level}

        frames = [torch.empty((v.height_px, v.width_px, 4), dtype=torch.uint8, device="cuda") for v in views]
        outs = []
        for f in frames:
            o = qb.Outputs()
            o.rgba8 = f.data_ptr()
            outs.append(o)
        # rays of a frame (the same for every arm: same pixels)
        flags = [torch.empty((v.height_px, v.width_px), dtype=torch.int32, device="cuda") for v in views]
        inst = []
        for f, fl in zip(frames, flags):
            o = qb.Outputs()
            o.rgba8, o.flags = f.data_ptr(), fl.data_ptr()
            inst.append(o)
        ctx.render_views(views, inst, on_device=True)
        torch.cuda.synchronize()
        rays = sum(count_rays(fl.cpu().numpy().view(np.uint32)) for fl in flags)
        out["rays_per_frame"] = rays

        mlp_kw = dict(two_pass=True, proposals=lib.PROPOSE_MLP, proposal_level=args.proposal_level)
        # learned: schedule and proposal settings (gate with "off", count,
        # level) tuned on the frame; learned_fixed: the same schedule with
        # the default proposal settings (gate 500, 3 proposals, level 8)
        arms = [("plain_fused", {}, 1), ("plain_two_pass", {"two_pass": True}, 1), ("learned", mlp_kw, 1),
                ("learned_fixed", mlp_kw, 1), ("plain_simple", {}, 0)]
        base = (ctx.get_option(lib.OPT_TILE_WIDTH), ctx.get_option(lib.OPT_BLOCKS_PER_SM),
                ctx.get_option(lib.OPT_SERVICE_MIN))
        fixed = {lib.OPT_PROPOSAL_GATE: 500, lib.OPT_PROPOSAL_COUNT: 3, lib.OPT_PROPOSAL_LEVEL: 8}
        res = {}
        for name, kw, persistent in arms:
            ctx.set_option(lib.OPT_PERSISTENT, persistent)
            if name == "learned_fixed":
                for k, v in fixed.items():
                    ctx.set_option(k, v)
                tuning = {"schedule": "as learned", "proposal_gate": 500, "proposal_count": 3, "proposal_level": 8}
            else:
                ctx.set_option(lib.OPT_TILE_WIDTH, base[0])
                ctx.set_option(lib.OPT_BLOCKS_PER_SM, base[1])
                ctx.set_option(lib.OPT_SERVICE_MIN, base[2])
                tuning = ctx.autotune(views, outs, reps=3, **kw) if args.autotune else None
            g = ctx.graph_capture(views, outs, **kw)
            ms = time_steps(g.launch, stream, flush, args.warmup, args.steps)
            g.close()
            # this arm's pixels for the parity sample
            chk = {k: [] for k in ("rgba8", "flags", "leaf")}
            couts = []
            for v in views:
                t = {"rgba8": torch.empty((v.height_px, v.width_px, 4), dtype=torch.uint8, device="cuda"),
                     "flags": torch.empty((v.height_px, v.width_px), dtype=torch.int32, device="cuda"),
                     "leaf": torch.empty((v.height_px, v.width_px, 4), dtype=torch.int32, device="cuda")}
                o = qb.Outputs()
                o.rgba8, o.flags, o.leaf = t["rgba8"].data_ptr(), t["flags"].data_ptr(), t["leaf"].data_ptr()
                for k in chk:
                    chk[k].append(t[k])
                couts.append(o)
            stats = ctx.render_views_ex(views, couts, True, **kw)
            torch.cuda.synchronize()
            frame = [{k: chk[k][i].cpu().numpy() for k in chk} for i in range(len(views))]
            res[name] = {"mrays": rays / (statistics.mean(ms) / 1000.0) / 1e6, "ms_per_frame": statistics.mean(ms),
                         "step_ms": [round(x, 4) for x in ms], "tuning": tuning, "frame": frame, "stats": stats}
        ctx.set_option(lib.OPT_PERSISTENT, 1)
        # the oracle on a seeded pixel sample, compared with every arm
        sample = cpu_sample(scene, views, budget_s=args.proposal_cpu_seconds, seed=31,
                            gpu_frames=res["plain_fused"]["frame"])
        kept = sample.pop("kept")
        for name, r in res.items():
            n = bad8 = badf = badl = 0
            for vi, px, py, ref in kept:
                g = r["frame"][vi]
                n += px.size
                bad8 += int((g["rgba8"][py, px] != ref["rgba8"]).any(axis=-1).sum())
                badf += int((g["flags"][py, px].view(np.uint32) != ref["flags"]).sum())
                gl = g["leaf"][py, px]
                # a proven pixel's shadow-leaf slot reads -2 (the plain walk's
                # leaf was not computed); every other slot must match
                skip = gl == -2
                skip[:, :2] = False
                badl += int(((gl != ref["leaf"]) & ~skip).any(axis=-1).sum())
            r["parity_sample"] = {"pixels": n, "rgba8_mismatch": bad8, "flags_mismatch": badf,
                                  "leaf_mismatch": badl}
            del r["frame"]
        two = res["plain_two_pass"]["stats"]
        for name in ("learned", "learned_fixed"):
            m = res[name]["stats"]
            vis = m["shadow_visits"] + m["proposal_visits"]
            res[name]["proposals"] = {
                "tried": m["proposals_tried"], "proven": m["proposals_proven"],
                "hit_rate": m["proposals_proven"] / max(1, m["proposals_tried"]),
                "shadow_visits": vis, "visits_saved_frac": 1.0 - vis / max(1, two["shadow_visits"])}
        for r in res.values():
            del r["stats"]
        out["arms"] = res
        ms_learned = res["learned"]["ms_per_frame"]
        tuned_gate = (res["learned"]["tuning"] or {}).get("proposal_gate")
        out.update({
            "speedup_vs_plain_fused": res["plain_fused"]["ms_per_frame"] / ms_learned,
            "speedup_vs_plain_two_pass": res["plain_two_pass"]["ms_per_frame"] / ms_learned,
            "speedup_vs_plain_simple": res["plain_simple"]["ms_per_frame"] / ms_learned,
            "learned_fixed_speedup_vs_plain_two_pass": res["plain_two_pass"]["ms_per_frame"]
            / res["learned_fixed"]["ms_per_frame"],
            "persistent_speedup_vs_plain_simple": res["plain_simple"]["ms_per_frame"] / res["plain_fused"]["ms_per_frame"],
            "network_switched_off_by_autotuner": tuned_gate == 1000,
            "shadow_rays": two["shadow_rays"], "shadow_visits_plain": two["shadow_visits"],
            "cpu_oracle": {k: v for k, v in sample.items() if k not in ("seconds", "rays", "parity")},
        })
    finally:
        ctx.close()
    return out


def flare_borderline(ctx, views, ulps: int = 2) -> dict:
    """Pixels whose flare test (acos(cos) < 0.02, evaluated as cos above the
    largest float not above cos(0.02)) sits within `ulps` floats of its
    threshold, over every pixel of the views, from the kernels' own camera
    rays: the pixels where a GL driver's acos could decide otherwise."""
    import torch
    within = near = 0
    for v in views:
        n = v.width_px * v.height_px
        idx = torch.arange(n, dtype=torch.int32, device="cuda")
        px = (idx % v.width_px).contiguous()
        py = (idx // v.width_px).contiguous()
        out = torch.empty((n, 4), dtype=torch.float32, device="cuda")
        ctx.camera_rays_device(v, px.data_ptr(), py.data_ptr(), n, out.data_ptr())
        torch.cuda.synchronize()
        cosv = out[:, 3].contiguous()
        thr = torch.tensor([v.flare_cos], dtype=torch.float32, device="cuda")
        within += int(((cosv > thr) & (cosv <= 1.0)).sum().item())
        d = (cosv.view(torch.int32).to(torch.int64) - thr.view(torch.int32).to(torch.int64)).abs()
        near += int((d <= ulps).sum().item())
    return {"pixels_in_flare_cone": within, "borderline_pixels": near, "ulps": ulps}


def proposal_sweep(ctx, qb, views, outs, stream, update, args):
    """Where the network's proposals could pay and why they do not: per cell
    level, gate and proposal count, the tries, proofs, hit rate, node visits
    per try (the cost of a failed try) against the plain shadow-walk visits a
    proof avoids, and the eager two-pass frame time; and the same for perfect
    proposals (the first leaf a logged plain render of the same frame found),
    the ceiling of any exact proposal. One frame (the first timed pose of
    the character, when there is one)."""
    import torch
    lib = qb._lib
    update(args.warmup)
    keep = {o: ctx.get_option(o) for o in (lib.OPT_PROPOSAL_GATE, lib.OPT_PROPOSAL_COUNT, lib.OPT_PROPOSAL_LEVEL)}
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]

    def frame(kw):
        ms = []
        stats = None
        for r in range(4):
            ev[0].record(stream)
            stats = ctx.render_views_ex(views, outs, True, **kw)
            ev[1].record(stream)
            torch.cuda.synchronize()
            if r:
                ms.append(ev[0].elapsed_time(ev[1]))
        return stats, statistics.median(ms)

    plain, plain_ms = frame({"two_pass": True})
    rows = []

    def row(source, gate, count, level, st, ms):
        tried, proven = st["proposals_tried"], st["proposals_proven"]
        avoided = plain["shadow_visits"] - st["shadow_visits"]
        rows.append({"source": source, "gate": gate, "count": count, "level": level, "tried": tried,
                     "proven": proven, "hit_rate": proven / max(1, tried),
                     "visits_per_try": st["proposal_visits"] / max(1, tried),
                     "plain_visits_avoided_per_proof": avoided / max(1, proven),
                     "shadow_visits_vs_plain": (st["shadow_visits"] + st["proposal_visits"])
                     / max(1, plain["shadow_visits"]),
                     "ms": ms, "speedup_vs_plain_two_pass": plain_ms / ms})

    for level in (5, 6, 7, 8):
        for gate in (500, 900):
            for count in (1, 3):
                ctx.set_option(lib.OPT_PROPOSAL_GATE, gate)
                ctx.set_option(lib.OPT_PROPOSAL_COUNT, count)
                ctx.set_option(lib.OPT_PROPOSAL_LEVEL, level)
                st, ms = frame({"two_pass": True, "proposals": lib.PROPOSE_MLP})
                row("network", gate, count, level, st, ms)
    if len(views) <= 32:  # the render log covers one launch of views
        ctx.render_views_ex(views, outs, True, two_pass=True, log=True)
        for level in (5, 6, 8):
            st, ms = frame({"two_pass": True, "proposals": lib.PROPOSE_LOGGED, "proposal_level": level})
            row("logged (perfect)", None, 1, level, st, ms)
    for o, v in keep.items():
        ctx.set_option(o, v)
    return {"plain_two_pass_ms": plain_ms, "shadow_rays": plain["shadow_rays"],
            "shadow_visits_plain": plain["shadow_visits"], "rows": rows,
            "timing": "eager two-pass frames, median of 3 after one untimed"}


def measure_paths(ctx, scene, stream, hbm_gbs: float) -> dict:
    """The traversal's other clients and producers on the bench's static
    scene, each on device arrays timed with CUDA events, beside the oracle's
    CPU version of the same work on a sample:
    - ray queries (qbc_trace_rays; oracle: qbo_trace on all host threads),
      8M seeded rays from inside the basecube; the oracle's status, leaf and
      model index must equal the GPU's on its sample;
    - the bulk build of the static tree from all points (qbc_build_tree;
      oracle: octree_insert_point in order, one thread, on a prefix of the
      points); the node count must equal the host producer's;
    - static edits, octree_remove_point of 1 % of the points in order
      (qbc_tree_remove_points; oracle: the same sequence on a copy of the
      node array, one thread); model and parent indices must be equal.
    The ray queries' algorithmic bytes count 32 B per node visit and 28 B
    per leaf hit (the leaf-box words are not counted: a lower bound)."""
    import ctypes as C
    import torch
    import qubatron_gb300 as qb
    from oracle import qbo
    spec = scene.spec
    S, L = float(spec.basesize), int(spec.levels)
    threads = os.cpu_count() or 1

    def timed(fn, reps=3, setup=None):
        ts = []
        for r in range(reps + 1):
            if setup:
                setup()
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            b.synchronize()
            if r:
                ts.append(a.elapsed_time(b))
        return statistics.median(ts)

    res = {}
    # -- ray queries --
    n = 8 << 20
    gen = torch.Generator(device="cuda").manual_seed(5)
    pos = (torch.rand((n, 3), generator=gen, device="cuda") * S).contiguous()
    d = torch.randn((n, 3), generator=gen, device="cuda")
    d = (d / d.norm(dim=1, keepdim=True)).contiguous()
    status = torch.empty(n, dtype=torch.int32, device="cuda")
    leaf = torch.empty((n, 2), dtype=torch.int32, device="cuda")
    model = torch.empty((n, 2), dtype=torch.int32, device="cuda")
    visits = torch.empty((n, 2), dtype=torch.int32, device="cuda")
    hits = qb._lib.RayHits(status.data_ptr(), leaf.data_ptr(), model.data_ptr(), None, None, None,
                           visits.data_ptr())
    bc = (C.c_float * 4)(0.0, S, S, S)

    def query():
        qb._lib.check(ctx._lib.qbc_trace_rays(ctx.handle, C.c_void_p(pos.data_ptr()), C.c_void_p(d.data_ptr()), n,
                                              bc, L, C.byref(hits), 1))

    ms = timed(query)
    n_vis = int(visits.to(torch.int64).sum())
    n_leaf = int((status == 1).sum())
    alg = 32.0 * n_vis + 28.0 * n_leaf
    k = 1 << 18
    sc = qbo.Scene(scene.nodes, scene.colors, scene.normals)
    hp, hd = pos[:k].cpu().numpy(), d[:k].cpu().numpy()
    t0 = time.perf_counter()
    cpu = qbo.trace_rays(sc, (0.0, S, S, S), L, hp, hd, threads)
    cpu_s = time.perf_counter() - t0
    bad = int((cpu["status"] != status[:k].cpu().numpy()).sum()
              + (cpu["leaf"] != leaf[:k].cpu().numpy()).any(axis=1).sum()
              + (cpu["model"] != model[:k].cpu().numpy()).any(axis=1).sum())
    res["ray_queries"] = {
        "rays": n, "ms": round(ms, 3), "mrays_per_s": n / ms / 1e3, "leaf_hits": n_leaf, "node_visits": n_vis,
        "roofline": {"bound": "hbm", "achieved": alg / (ms / 1e3) / 1e9, "peak": hbm_gbs, "unit": "GB/s",
                     "frac": alg / (ms / 1e3) / 1e9 / hbm_gbs,
                     "algorithmic": "32 B per node visit + 28 B per leaf hit (leaf-box words not counted)"},
        "cpu_baseline": {"value": k / cpu_s / 1e6, "unit": "Mrays/s", "cores": threads, "kind": "port",
                         "sample": f"the first {k} rays"},
        "parity_sample": {"rays": k, "mismatches": bad, "streams": "status, leaf, model"}}
    del pos, d, status, leaf, model, visits
    # -- bulk build of the static tree --
    pts = torch.from_numpy(np.ascontiguousarray(scene.points, np.float32)).cuda()
    npts = int(pts.shape[0])

    def build():
        ctx.build_tree(False, (pts.data_ptr(), npts), S, L, count=False)

    ms = timed(build)
    nodes = ctx.tree_nodes(0)
    m = min(npts, 2_000_000)
    t0 = time.perf_counter()
    qbo.build_tree(scene.points[:m], S, L)
    cpu_s = time.perf_counter() - t0
    res["bulk_build"] = {
        "points": npts, "ms": round(ms, 3), "mpoints_per_s": npts / ms / 1e3, "nodes": nodes,
        "nodes_equal_host_producer": nodes == int(scene.nodes.shape[0]),
        "cpu_baseline": {"value": m / cpu_s / 1e6, "unit": "Mpoints/s", "cores": 1, "kind": "port",
                         "sample": f"the first {m} points into an empty tree"}}
    # -- static edits: remove 1 % of the points, in a seeded order --
    rng = np.random.default_rng(9)
    sel = np.ascontiguousarray(scene.points[rng.choice(npts, npts // 100, replace=False)], np.float32)
    nsel = sel.shape[0]
    sel_d = torch.from_numpy(sel).cuda()
    mod = torch.empty(nsel, dtype=torch.int32, device="cuda")
    par = torch.empty(nsel, dtype=torch.int32, device="cuda")
    removed = C.c_int64()
    i32 = C.POINTER(C.c_int32)

    def remove():
        fp = C.cast(C.c_void_p(sel_d.data_ptr()), qb._lib.c_float_p)
        qb._lib.check(ctx._lib.qbc_tree_remove_points(ctx.handle, 0, fp, nsel, S, L, 1,
                                                      C.cast(C.c_void_p(mod.data_ptr()), i32),
                                                      C.cast(C.c_void_p(par.data_ptr()), i32), C.byref(removed)))

    ms = timed(remove, setup=build)  # each edit on a freshly built tree
    host = np.ascontiguousarray(scene.nodes, np.int32).copy()
    t0 = time.perf_counter()
    cmod, cpar = qbo.remove_points(host, sel, S, L)
    cpu_s = time.perf_counter() - t0
    res["static_edits"] = {
        "points_removed": nsel, "ms": round(ms, 3), "mpoints_per_s": nsel / ms / 1e3, "removed": removed.value,
        "cpu_baseline": {"value": nsel / cpu_s / 1e6, "unit": "Mpoints/s", "cores": 1, "kind": "port",
                         "sample": f"all {nsel} removals on a copy of the node array"},
        "parity": {"model_and_parent_equal": bool(np.array_equal(cmod, mod.cpu().numpy())
                                                  and np.array_equal(cpar, par.cpu().numpy()))}}
    ctx.build_tree(False, (pts.data_ptr(), npts), S, L)  # leave the tree whole
    torch.cuda.synchronize()
    return res


def run_gpu(args):
    import torch
    import qubatron_gb300 as qb
    from qubatron_gb300 import replicas

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    w, scene, views, character, prep_s = prepare(WORKLOAD, host_nodes=False)

    ctx = qb.OctreeGLC(local)
    # a dedicated stream: the library and the timing events must share it
    # (torch's default stream is the legacy NULL stream, which the library
    # does not take as a launch stream)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    ctx.upload_model(False, scene.colors, scene.normals)
    if scene.nodes is not None:
        ctx.upload_octree(False, scene.nodes)
        n_nodes = int(scene.nodes.shape[0])
    else:
        # octree_insert_point numbering, built on the GPU
        n_nodes = ctx.build_tree(False, scene.points, scene.spec.basesize, scene.spec.levels)
        torch.cuda.synchronize()
    if args.service_min:
        ctx.set_option(qb._lib.OPT_SERVICE_MIN, args.service_min)
    if args.tile_width:
        ctx.set_option(qb._lib.OPT_TILE_WIDTH, args.tile_width)
    if args.blocks_per_sm:
        ctx.set_option(qb._lib.OPT_BLOCKS_PER_SM, args.blocks_per_sm)
    if args.split_trees >= 0:
        ctx.set_option(qb._lib.OPT_SPLIT_TREES, args.split_trees)

    def render_plain(v, o, dev):
        ctx.render_views(v, o, on_device=dev)

    def render_two_pass(v, o, dev):
        ctx.render_views_ex(v, o, dev, two_pass=True)

    mlp_kw = dict(two_pass=True, proposals=qb._lib.PROPOSE_MLP, proposal_level=args.proposal_level)

    def render_mlp(v, o, dev):
        ctx.render_views_ex(v, o, dev, **mlp_kw)

    graphs = []

    def as_graph(kw):
        """The frame as a CUDA graph: each step is one qbc_graph_launch into
        the device outputs; with a character the graph also holds the
        frame's dynamic update (skin, rebuild, normals), and a step writes
        the frame's bones before the launch."""
        g = ctx.graph_capture_dynamic(chars.update, views, outs, **kw) if chars else ctx.graph_capture(views, outs, **kw)
        graphs.append(g)
        fn = lambda v, o, dev: g.launch()  # noqa: E731
        fn.graph = True
        return fn

    # device outputs
    frames = [torch.empty((v.height_px, v.width_px, 4), dtype=torch.uint8, device="cuda") for v in views]
    outs = []
    for f in frames:
        o = qb.Outputs()
        o.rgba8 = f.data_ptr()
        outs.append(o)

    n_frames = args.warmup + args.steps
    chars = CharacterFrames(ctx, character, n_frames) if character is not None else None

    def update(frame, eager=True):
        """The frame's dynamic basecube: the whole update, or (graph steps)
        only its bones."""
        if chars:
            chars.apply(frame) if eager else chars.set_bones(frame)

    render = render_plain
    training = None
    if w.train_poses:
        update(0)
        # occluder-proposal network: log the plain shadow walks of the
        # training poses, train on them (both untimed), render the held-out
        # poses with its proposals
        from qubatron_gb300 import scenes as _sc
        tv = _sc.train_views(w)
        t0 = time.time()
        samples = 0
        for i in range(0, len(tv), 32):
            samples = ctx.proposal_collect(tv[i:i + 32])
        collect_s = time.time() - t0
        t0 = time.time()
        st = ctx.proposal_train(steps=args.train_steps, batch=8192, lr=2e-3, seed=1)
        torch.cuda.synchronize()
        training = {"poses": len(tv), "pose_size": "%dx%d" % w.train_size, "samples": samples,
                    "occluded": st["occluded"], "steps": args.train_steps, "batch": 8192,
                    "loss_first": st["loss_first"], "loss_last": st["loss_last"],
                    "collect_s": round(collect_s, 2), "train_s": round(time.time() - t0, 2),
                    "gate_per_mille": args.proposal_gate, "proposal_level": args.proposal_level}
        ctx.set_option(qb._lib.OPT_PROPOSAL_GATE, args.proposal_gate)
        ctx.set_option(qb._lib.OPT_PROPOSAL_COUNT, args.proposal_count)
        training["proposal_count"] = args.proposal_count
        render = render_mlp

    tuning = None
    if args.autotune and not (args.service_min or args.tile_width or args.blocks_per_sm):
        # tuning options (service threshold, warp tile, blocks per SM) picked
        # by timing this frame; untimed
        update(0)
        # very large frames: tune on the first views holding ~100M pixels
        # (same sizes and scene; enough pixels per launch that the fixed
        # costs of a launch, e.g. a split frame's second tail, weigh as in
        # the whole frame)
        k, px = 0, 0
        while k < len(views) and px < 100_000_000:
            px += views[k].width_px * views[k].height_px
            k += 1
        tuning = ctx.autotune(views[:k], outs[:k], reps=3, **(mlp_kw if training is not None else {}))
        tuning["views_timed"] = k
        torch.cuda.synchronize()

    use_graph = args.graph
    if use_graph:
        render = as_graph(mlp_kw if training is not None else {})

    # untimed instrumented passes: rays cast and node visits of every timed
    # frame (a static scene needs one)
    flags = [torch.empty((v.height_px, v.width_px), dtype=torch.int32, device="cuda") for v in views]
    visits = [torch.empty((v.height_px, v.width_px, 4), dtype=torch.int32, device="cuda") for v in views]
    inst = []
    for f, fl, vi in zip(frames, flags, visits):
        o = qb.Outputs()
        o.rgba8 = f.data_ptr()
        o.flags = fl.data_ptr()
        o.visits = vi.data_ptr()
        inst.append(o)
    frame_rays, frame_bytes, frame_visits, frame_words = [], [], [], []
    for k in range(args.steps if chars else 1):
        update(args.warmup + k)
        words_k = ctx.render_views_ex(views, inst, on_device=True)["box_words"]
        torch.cuda.synchronize()
        rays_k, vis_k, leaves_k = 0, 0, 0
        for fl, vi in zip(flags, visits):
            f = fl.cpu().numpy().view(np.uint32)
            rays_k += count_rays(f)
            leaves_k += int((f & 1).sum()) + int(((f >> 3) & 1).sum())
            vis_k += int(vi.to(torch.int64).sum().item())
        pixels = sum(v.width_px * v.height_px for v in views)
        frame_rays.append(rays_k)
        frame_visits.append(vis_k)
        frame_words.append(words_k)
        frame_bytes.append(vis_k * BYTES_PER_VISIT + words_k * BYTES_PER_BOX_WORD + leaves_k * BYTES_PER_LEAF
                           + pixels * BYTES_PER_PIXEL_OUT)
    if not chars:
        frame_rays *= args.steps
        frame_bytes *= args.steps
    rays = statistics.mean(frame_rays)
    alg_bytes = statistics.mean(frame_bytes)
    del flags, visits

    flush = torch.empty(2 * L2_BYTES, dtype=torch.uint8, device="cuda")

    def timed(render_fn):
        eager = not getattr(render_fn, "graph", False)
        for f in range(args.warmup):
            update(f, eager)
            render_fn(views, outs, True)
        torch.cuda.synchronize()
        l0 = ctx.launch_count()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        replicas.barrier()
        torch.cuda.synchronize()
        with ClockSampler(local) as clk:
            for k in range(args.steps):
                flush.zero_()
                ev[k][0].record(stream)
                update(args.warmup + k, eager)
                render_fn(views, outs, True)
                ev[k][1].record(stream)
            torch.cuda.synchronize()
        replicas.barrier()
        return [a.elapsed_time(b) for a, b in ev], ctx.launch_count() - l0, clk

    step_ms, launches, clk = timed(render)
    # replicas: every rank renders the whole workload; the job's throughput
    # is all ranks' rays over the slowest rank's time
    rate, slowest_s = replicas.job_throughput(sum(frame_rays), sum(step_ms) / 1000.0, device="cuda")
    value = rate / 1e6
    ms = 1000.0 * slowest_s / len(step_ms)

    proposal = None
    if training is not None:
        # the same frames without the network (fused kernel, and the same
        # two-pass pipeline), and the proposal statistics of one frame
        plain_ms, _, _ = timed(as_graph({}) if use_graph else render_plain)
        two_ms, _, _ = timed(as_graph({"two_pass": True}) if use_graph else render_two_pass)
        st_mlp = ctx.render_views_ex(views, outs, True, two_pass=True, proposals=qb._lib.PROPOSE_MLP,
                                     proposal_level=args.proposal_level)
        st_two = ctx.render_views_ex(views, outs, True, two_pass=True)
        vis_mlp = st_mlp["shadow_visits"] + st_mlp["proposal_visits"]
        mrays = lambda xs: sum(frame_rays) / (sum(xs) / 1000.0) / 1e6
        proposal = {
            "training": training,
            "plain_fused_mrays": mrays(plain_ms), "plain_two_pass_mrays": mrays(two_ms), "mlp_mrays": value,
            "speedup_vs_plain_fused": statistics.mean(plain_ms) / statistics.mean(step_ms),
            "speedup_vs_plain_two_pass": statistics.mean(two_ms) / statistics.mean(step_ms),
            "shadow_rays": st_two["shadow_rays"], "proposals_tried": st_mlp["proposals_tried"],
            "proposals_proven": st_mlp["proposals_proven"],
            "hit_rate": st_mlp["proposals_proven"] / max(1, st_mlp["proposals_tried"]),
            "shadow_visits_plain": st_two["shadow_visits"], "shadow_visits_mlp": vis_mlp,
            "visits_saved_frac": 1.0 - vis_mlp / max(1, st_two["shadow_visits"]),
        }

    if training is not None and args.proposal_sweep:
        proposal["sweep"] = proposal_sweep(ctx, qb, views, outs, stream, update, args)

    # the same frames on the plain one-thread-per-pixel schedule (no
    # persistent queue, no batched ray starts), same tuning otherwise
    ctx.set_option(qb._lib.OPT_PERSISTENT, 0)
    simple_ms, _, _ = timed(as_graph({}) if use_graph else render_plain)
    ctx.set_option(qb._lib.OPT_PERSISTENT, 1)
    plain_simple = {"mrays": sum(frame_rays) / (sum(simple_ms) / 1000.0) / 1e6,
                    "ms_per_step": statistics.mean(simple_ms),
                    "speedup_of_value": statistics.mean(simple_ms) / statistics.mean(step_ms),
                    "schedule": "one thread per pixel for its whole life, one warp per 32-pixel tile "
                                "(QBC_OPT_PERSISTENT 0)"}

    update_ms = None
    if chars:
        # the dynamic-tree update alone (skin + rebuild + normals), untimed above
        ue = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(3)]
        for k in range(3):
            ue[k][0].record(stream)
            update(args.warmup + k % args.steps)
            ue[k][1].record(stream)
        torch.cuda.synchronize()
        update_ms = statistics.mean(a.elapsed_time(b) for a, b in ue)

    e2e = None
    if not args.no_e2e:
        e2e = measure_e2e(ctx, views, rays, world, flush, args.steps,
                          (lambda k: update(args.warmup + k % args.steps)) if chars else None,
                          render_mlp if training is not None else render_plain,
                          chars.h2d_bytes if chars else 0)

    hbm, peak_kind = peaks()

    achieved = alg_bytes / (ms / 1000.0) / 1e9
    # DRAM traffic of the frame kernel: one ncu capture of a one-view case of
    # the same scene (profiles/), scaled to this launch by algorithmic bytes
    traffic, traffic_kind = None, None
    tpath = os.path.join(ROOT, "profiles", "render_kernel_traffic.json")
    if os.path.exists(tpath):
        with open(tpath) as f:
            t = json.load(f)
        if t.get("applies_to") == WORKLOAD:
            traffic = t["dram_bytes_per_launch_captured"] * alg_bytes / t["algorithmic_bytes_per_launch_captured"]
            traffic_kind = (f"ncu dram__bytes of {t['captured_on']} ({t['dram_bytes_per_launch_captured']} B), "
                            "scaled by algorithmic bytes to this launch")

    line = {
        "metric": "primary+shadow Mrays/s", "value": value, "unit": "Mrays/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene)",
        "config": workload_config(w, scene, n_nodes, views),
        "run": {"rays_per_step": rays, "nominal_2wh_rays_per_step": 2 * pixels, "dynamic_update_ms": update_ms,
                "prep_seconds": round(prep_s, 1)},
        "e2e": e2e,
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": traffic, "traffic_kind": traffic_kind, "peak_kind": f"{peak_kind} (burst copy)",
                     "algorithmic_bytes_per_launch": alg_bytes,
                     "node_visits_per_launch": statistics.mean(frame_visits),
                     "box_words_per_launch": statistics.mean(frame_words)},
        "clocks": clk.summary(),
        "step_ms": [round(x, 4) for x in step_ms],
    }
    line["plain_simple"] = plain_simple
    line["flare_test"] = flare_borderline(ctx, views)
    if proposal is not None:
        line["run"]["per_step"] = "two-pass render with occluder-network proposals (network evaluated every step)"
        line["proposal"] = proposal
    elif not args.no_proposal_block and world == 1:
        # the metric's learned-vs-plain comparison, on its own workload
        line["proposal"] = proposal_comparison(args, local, stream, flush)
    line["run"]["launch"] = "CUDA graph replay (qbc_graph_launch)" if use_graph else "eager (qbc_render_views*)"
    line["run"]["tuning"] = tuning
    for g in graphs:
        g.close()
    if rank == 0 and not args.no_cpu_baseline:
        if scene.nodes is None:
            scene.nodes = ctx.download_tree(False)  # the GPU-built tree, for the host oracle
        # the frame the CPU sample renders (the character's pose of frame
        # `warmup`), once more on the GPU with the streams the check compares
        update(args.warmup)
        chk, couts = [], []
        for v in views:
            t = {"rgba8": torch.empty((v.height_px, v.width_px, 4), dtype=torch.uint8, device="cuda"),
                 "flags": torch.empty((v.height_px, v.width_px), dtype=torch.int32, device="cuda"),
                 "leaf": torch.empty((v.height_px, v.width_px, 4), dtype=torch.int32, device="cuda")}
            o = qb.Outputs()
            o.rgba8, o.flags, o.leaf = t["rgba8"].data_ptr(), t["flags"].data_ptr(), t["leaf"].data_ptr()
            chk.append(t)
            couts.append(o)
        ctx.render_views(views, couts, on_device=True)
        torch.cuda.synchronize()
        gpu_frames = [{k: a.cpu().numpy() for k, a in t.items()} for t in chk]
        del chk
        res = cpu_sample(scene, views, budget_s=args.cpu_seconds, character=character, frame=args.warmup,
                         gpu_frames=gpu_frames)
        res.pop("kept", None)
        line["parity_sample"] = res.pop("parity")
        line["parity_sample"]["streams"] = "rgba8, flags, leaf (GPU frame vs the oracle on the CPU sample's pixels)"
        line["cpu_baseline"] = {k: v for k, v in res.items() if k not in ("seconds", "rays")}
    if args.paths and world == 1 and scene.nodes is not None and character is None:
        # last: it rebuilds and edits the static tree
        line["paths"] = measure_paths(ctx, scene, stream, peaks()[0])
    ctx.close()
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--service-min", type=int, default=0, help="set the service threshold (no autotune)")
    ap.add_argument("--tile-width", type=int, default=0, help="set the warp tile width 4/8/16/32 (no autotune)")
    ap.add_argument("--blocks-per-sm", type=int, default=0, help="set render blocks per SM (no autotune)")
    ap.add_argument("--paths", action="store_true",
                    help="also time ray queries, the GPU bulk build and static edits on the scene (with the oracle)")
    ap.add_argument("--split-trees", type=int, default=-1, choices=[-1, 0, 1],
                    help="two-tree fused frames: 1 one-tree + two-tree launch, 0 one launch (-1: library default)")
    ap.add_argument("--workload", default=None)
    ap.add_argument("--train-steps", type=int, default=4000, help="occluder-network training steps")
    ap.add_argument("--no-autotune", dest="autotune", action="store_false",
                    help="keep the default tuning options instead of autotuning them on the frame")
    ap.add_argument("--no-graph", dest="graph", action="store_false",
                    help="time eager launches instead of CUDA graph replays of the frame")
    ap.add_argument("--proposal-gate", type=int, default=500, help="occlusion probability (per mille) to try")
    ap.add_argument("--proposal-level", type=int, default=0,
                    help="octree level of the proposed cells (0: the context's, swept by the autotuner)")
    ap.add_argument("--proposal-count", type=int, default=3, help="network proposals tried per pixel (1..3)")
    ap.add_argument("--proposal-sweep", action="store_true",
                    help="network workloads: per level, gate and count, the proposals' hit rate and cost")
    ap.add_argument("--no-proposal-block", action="store_true",
                    help="skip the learned-vs-plain comparison on the proposal workload")
    ap.add_argument("--proposal-cpu-seconds", type=float, default=4.0,
                    help="oracle time for the proposal comparison's parity sample")
    args = ap.parse_args()
    global WORKLOAD
    if args.workload:
        WORKLOAD = args.workload
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
