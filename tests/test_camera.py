"""Ray generation pinned to the reference's own C quaternion code.

tests/golden/camera_quat.npz holds, for 88 cameras (the benchmark poses and
edge angles), the frame quaternions and 32 per-pixel camera rays that the
reference's src/mt_math/mt_quat.c computes (quat_from_axis_angle and
quat_rotate, the formulas of the shader's octree_fsh.c:381-395, applied as
main() does at octree_fsh.c:401-413). The library's uniform derivation, the
oracle and (tests/test_gpu_parity.py) the kernels' per-pixel rays must equal
them bit for bit."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, S


@pytest.fixture(scope="module")
def cams():
    return dict(np.load(os.path.join(GOLDEN, "camera_quat.npz")))


def camera_args(g, vi):
    sw, sh, q, focal, x, y, z = g["cam"][vi]
    ang = (float(g["angle"][vi][0]), float(g["angle"][vi][1]), 0.0)
    return float(sw), float(sh), (float(x), float(y), float(z)), ang, 0.0, int(q), 12, S, 0, float(focal)


def test_frame_quaternions_match_mt_quat(lib, oracle, cams):
    import qubatron_gb300 as qb
    for vi in range(cams["angle"].shape[0]):
        w, h, pos, ang, la, q, ml, bs, sh, f = camera_args(cams, vi)
        for v in (qb.view_setup(w, h, pos, ang, la, q, ml, bs, sh, f), oracle.view_setup(w, h, pos, ang, la, q, ml, bs, sh, f)):
            assert np.array(v.qz, np.float32).tobytes() == cams["qz"][vi].tobytes(), f"camera {vi}: qz"
            assert np.array(v.qx, np.float32).tobytes() == cams["qx"][vi].tobytes(), f"camera {vi}: qx"


def test_oracle_camera_rays_match_mt_quat(oracle, cams):
    for vi in range(cams["angle"].shape[0]):
        v = oracle.view_setup(*camera_args(cams, vi))
        m = cams["view"] == vi
        got = oracle.camera_rays(v, cams["px"][m], cams["py"][m])
        np.testing.assert_array_equal(got[:, :3].view(np.uint32), cams["csv"][m].view(np.uint32))


def test_reference_quaternions_cover_edge_angles(cams):
    # yaw of +-pi and pitch of +-1.5 are in the set; each camera has its
    # four corner pixels and its centre
    assert np.abs(cams["angle"][:, 0]).max() > 3.14 and np.abs(cams["angle"][:, 1]).max() >= 1.5
    assert cams["px"].size == 32 * cams["angle"].shape[0]
