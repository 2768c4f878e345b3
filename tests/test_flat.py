"""qmc flat model files: the library's reader (qbc_flat_read) against what
the reference's own model_load_flat (src/qubatron/model.c:53-111) read from
the same files (tests/golden/flat_small.npz, recorded by make_golden.py),
plus the size rules and errors. No GPU."""
import os

import numpy as np
import pytest

from conftest import ROOT

PREFIX = os.path.join(ROOT, "tests", "golden", "flat", "small")


def test_reader_matches_reference_loader():
    from qubatron_gb300.flatfile import read_flat
    ref = np.load(os.path.join(ROOT, "tests", "golden", "flat_small.npz"))
    got = read_flat(PREFIX)
    assert got["points"].shape == ref["points"].shape == (2000, 3)  # 7 trailing bytes ignored
    for k in ("points", "colors", "normals", "ranges"):
        assert np.array_equal(got[k].view(np.uint8), ref[k].view(np.uint8)), k
    assert got["ranges"].size == 120  # the partial int after the last triple is ignored


def test_round_trip_and_size_rules(tmp_path):
    from qubatron_gb300.flatfile import read_flat, write_flat
    rng = np.random.default_rng(3)
    p, n, c = (rng.uniform(0, 1800, (333, 3)).astype(np.float32) for _ in range(3))
    r = rng.integers(-5, 5000, 99).astype(np.int32)
    prefix = str(tmp_path / "m")
    write_flat(prefix, p, n, c, r)
    got = read_flat(prefix)
    for k, a in (("points", p), ("normals", n), ("colors", c), ("ranges", r)):
        assert np.array_equal(got[k], a), k
    # a normal file shorter than the point file: the rest reads as 0
    n[:100].tofile(prefix + ".nrm")
    got = read_flat(prefix)
    assert np.array_equal(got["normals"][:100], n[:100]) and not got["normals"][100:].any()
    # no range file requested
    assert read_flat(prefix, ranges=False)["ranges"].size == 0
    # empty model
    write_flat(prefix, np.zeros((0, 3)), np.zeros((0, 3)), np.zeros((0, 3)))
    got = read_flat(prefix)
    assert got["points"].shape == (0, 3) and got["ranges"].size == 0


def test_reader_errors(tmp_path):
    import ctypes as C
    import qubatron_gb300._lib as L
    from qubatron_gb300 import QbcError
    from qubatron_gb300.flatfile import paths, read_flat
    with pytest.raises(QbcError) as e:
        read_flat(str(tmp_path / "missing"))
    assert e.value.code == -6  # QBC_E_IO
    lib = L.load()
    p = [s.encode() for s in paths(PREFIX)]
    n, nr = C.c_int64(), C.c_int64()
    small = np.zeros((10, 3), np.float32)
    f = L.c_float_p
    rc = lib.qbc_flat_read(p[0], p[1], p[2], p[3], small.ctypes.data_as(f), small.ctypes.data_as(f),
                           small.ctypes.data_as(f), 10, C.byref(n), None, 0, C.byref(nr))
    assert rc == -1 and n.value == 2000  # capacity too small: QBC_E_ARG, counts still reported
    rc = lib.qbc_flat_read(p[0], p[1], p[2], p[3], small.ctypes.data_as(f), None, None, 10, C.byref(n), None, 0,
                           C.byref(nr))
    assert rc == -1
