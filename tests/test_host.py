"""Host-side checks that need no GPU: the C ABI loads and exports every
function include/qbcuda.h declares, the uniform derivation equals the
oracle's, and the node-array producer equals the reference's (via the
fixtures recorded from the reference's octree.c)."""
import hashlib
import os
import re

import numpy as np
import pytest

from conftest import LEVELS, ROOT, S


def declared_functions():
    text = open(os.path.join(ROOT, "include", "qbcuda.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(qbc_[a-z0-9_]+)\s*\(", text)))


def test_abi_exports_every_declared_function(lib):
    import qubatron_gb300._lib as L
    names = declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), f"{n} declared in qbcuda.h but not exported"
        assert n in L.SIGNATURES, f"{n} has no ctypes signature"


def test_abi_symbols_are_c_linkage():
    out = os.popen(f"nm -D --defined-only {os.path.join(ROOT, 'qubatron_gb300', '_build', 'libqbcuda.so')}").read()
    for n in declared_functions():
        assert re.search(rf"\bT {n}$", out, re.M), n


def test_struct_layouts_match_oracle(oracle):
    import ctypes as C
    import qubatron_gb300._lib as L
    assert C.sizeof(L.View) == C.sizeof(oracle.QboView) == 132
    assert [f[0] for f in L.View._fields_] == [f[0] for f in oracle.QboView._fields_]


@pytest.mark.parametrize("args", [
    (640, 480, (903.7, 421.3, 1702.9), (0.0, -0.3, 0.0), 0.0, 10, 12, 1800.0, 0, 415.69),
    (1200, 800, (700.0, 150.0, 350.0), (0.7, 0.1, 0.0), 1.3, 10, 12, 1800.0, 1, 0.0),
    (1200, 800, (700.0, 150.0, 350.0), (-2.0, -0.2, 0.0), 0.4, 7, 11, 1234.5, 0, 0.0),
    (1201, 799, (1.0, 2.0, 3.0), (3.0, 1.5, 0.0), -7.0, 3, 17, 100.0, 0, 0.0),
])
def test_view_setup_matches_oracle(lib, oracle, args):
    from qubatron_gb300 import view_setup
    a = view_setup(*args)
    b = oracle.view_setup(*args)
    assert a.to_bytes() == b.to_bytes()


def test_view_setup_reference_sizes(lib):
    """octree_glc.c:268-270: ow = width / (6 - quality/2), viewport (int)ow."""
    from qubatron_gb300 import view_setup
    v = view_setup(1200, 800, (0, 0, 0), (0, 0, 0), 0.0, 10, 12, S)
    assert (v.width_px, v.height_px, v.dim[0], v.dim[1]) == (1200, 800, 1200.0, 800.0)
    assert v.cfp[2] == 600.0  # (ow/2)/tan(pi/4) with tan(pi/4) rounding to 1
    v = view_setup(1200, 800, (0, 0, 0), (0, 0, 0), 0.0, 9, 12, S)
    assert (v.width_px, v.height_px) == (800, 533)
    assert v.light[:] == [420.0, 200.0, 680.0]


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).digest()


def test_scene_generator_is_deterministic(lib, floor50k, floor50k_scene):
    assert sha(floor50k_scene.points) == floor50k["points_sha256"].tobytes()


def test_producer_matches_reference(lib, floor50k, floor50k_scene):
    assert floor50k_scene.nodes.shape[0] == int(floor50k["n_nodes"])
    assert sha(floor50k_scene.nodes) == floor50k["nodes_sha256"].tobytes()


def test_producer_five_point(lib, five_point):
    from qubatron_gb300 import build_octree
    np.testing.assert_array_equal(build_octree(five_point["points"], S, LEVELS), five_point["nodes"])


def test_producer_paths_and_remove(lib, oracle, floor50k, floor50k_scene):
    from qubatron_gb300 import Octree
    pts = floor50k_scene.points
    t = Octree(S, LEVELS)
    t.insert_paths(oracle.point_octets(pts, S, LEVELS))
    assert sha(t.nodes) == floor50k["paths_sha256"].tobytes()
    t = Octree(S, LEVELS)
    t.insert_points(pts)
    out = [t.remove_point(pts[i]) for i in floor50k["remove_idx"]]
    np.testing.assert_array_equal(np.array(out, np.int32), floor50k["remove_out"])
    assert sha(t.nodes) == floor50k["removed_sha256"].tobytes()
    t.reset()
    assert len(t) == 1 and not t.nodes.any()


def test_producer_rejects_bad_points(lib):
    from qubatron_gb300 import Octree, QbcError
    t = Octree(S, LEVELS)
    with pytest.raises(QbcError):
        t.insert_points(np.array([[-1.0, 5.0, 5.0]], np.float32))
    with pytest.raises(QbcError):
        t.insert_points(np.array([[np.nan, 5.0, 5.0]], np.float32))
    with pytest.raises(QbcError):
        t.insert_paths(np.full((1, LEVELS), 9, np.int32))


def test_library_errors_without_gpu(lib):
    """Context creation reports an error code instead of crashing when no
    CUDA device is usable."""
    import ctypes as C
    h = C.c_void_p()
    rc = lib.qbc_create(0, C.byref(h))
    if rc == 0:
        lib.qbc_destroy(h)
        pytest.skip("a GPU is present")
    assert rc in (-1, -2)
    assert lib.qbc_last_error()


STRUCTS = [("View", "qbc_view"), ("Outputs", "qbc_outputs"), ("RayHits", "qbc_ray_hits"),
           ("RenderOpts", "qbc_render_opts"), ("RenderStats", "qbc_render_stats"), ("TuneResult", "qbc_tune_result"),
           ("TrainOpts", "qbc_train_opts"), ("TrainStats", "qbc_train_stats"), ("SceneDesc", "qbc_scene_desc")]


def test_ctypes_structs_match_header(tmp_path):
    """Size and every field offset of each ctypes mirror equal the C
    compiler's layout of the header's struct."""
    import ctypes as C
    import subprocess
    import qubatron_gb300._lib as L
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "qbcuda.h"', "int main(void) {"]
    for py, c in STRUCTS:
        lines.append(f'  printf("{py} size %zu\\n", sizeof({c}));')
        for f in getattr(L, py)._fields_:
            lines.append(f'  printf("{py} {f[0]} %zu\\n", offsetof({c}, {f[0]}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = {}
    for ln in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines():
        py, key, val = ln.split()
        got[py, key] = int(val)
    for py, _ in STRUCTS:
        cls = getattr(L, py)
        assert got[py, "size"] == C.sizeof(cls), py
        for f in cls._fields_:
            assert got[py, f[0]] == getattr(cls, f[0]).offset, (py, f[0])
