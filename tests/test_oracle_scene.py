"""The oracle's own workload builders against the library's: the benchmark's
reference arm builds its scene, node array and uniforms with the oracle alone,
so these must equal what the GPU arm builds with libqbcuda, bit for bit."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import LEVELS, ROOT, S


@pytest.mark.parametrize("name", ["floor1m", "room20m", "house90m"])
def test_scene_generator_matches_library(lib, oracle, name):
    from qubatron_gb300 import scenes
    spec = scenes.scaled_spec(name, 60_000)
    mine = scenes.generate_points(spec)
    theirs = oracle.scene_generate(spec.kind, spec.n_points, spec.seed, spec.n_boxes, spec.box, spec.n_spheres,
                                   spec.sphere, spec.color_noise, spec.basesize, spec.levels)
    for a, b, what in zip(mine, theirs, ("points", "normals", "colours")):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), f"{name}: {what} differ"


def test_bulk_producer_matches_library(lib, oracle):
    from qubatron_gb300 import scenes
    spec = scenes.scaled_spec("room20m", 80_000)
    pts = scenes.generate_points(spec)[0]
    # shuffled, with duplicates: insertion order decides the numbering
    rng = np.random.default_rng(3)
    pts = np.concatenate([pts, pts[:500]])[rng.permutation(pts.shape[0] + 500)]
    np.testing.assert_array_equal(oracle.build_tree(pts, S, LEVELS), scenes.build_octree(pts, S, LEVELS))


def test_view_setup_matches_library(lib, oracle):
    import qubatron_gb300 as qb
    from qubatron_gb300 import scenes
    for w in (scenes.WORKLOADS["room20m_1920x1080x16"], scenes.WORKLOADS["floor1m_char2m_mixed_x64"]):
        a = scenes.workload_views(w)
        b = scenes.workload_views(w, view_setup=oracle.view_setup)
        assert [bytes(memoryview(x).cast("B")) for x in a] == [x.to_bytes() for x in b]
    v1 = qb.view_setup(700.0, 500.0, (12.5, 900.0, 33.0), (2.9, -1.1, 0.0), 0.7, 3, 9, 1800.0, 1, 0.0)
    v2 = oracle.view_setup(700.0, 500.0, (12.5, 900.0, 33.0), (2.9, -1.1, 0.0), 0.7, 3, 9, 1800.0, 1, 0.0)
    assert bytes(memoryview(v1).cast("B")) == v2.to_bytes()


def test_reference_arm_maps_only_the_oracle(lib):
    """bench.py --impl reference on a small workload: its line names only
    oracle libraries, and its config equals the GPU arm's for the same
    workload (built here through libqbcuda's host producer)."""
    env = dict(os.environ)
    env.pop("RANK", None)
    env.pop("WORLD_SIZE", None)
    res = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload",
                          "floor1m_640x480", "--steps", "1", "--warmup", "3", "--cpu-seconds", "0.2"],
                         capture_output=True, text=True, timeout=600, env=env, cwd=ROOT)
    assert res.returncode == 0, res.stderr[-2000:]
    line = json.loads(res.stdout.strip().splitlines()[-1])
    assert line["libraries_mapped"] and all(x.startswith("oracle" + os.sep) for x in line["libraries_mapped"])
    sys.path.insert(0, ROOT)
    import bench
    w, scene, views, _, _ = bench.prepare("floor1m_640x480")
    assert line["config"] == bench.workload_config(w, scene, scene.nodes.shape[0], views)
