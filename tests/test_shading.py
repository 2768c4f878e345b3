"""The shading of octree_fsh.c:431-449 pinned to the reference's own C
vector helpers.

tests/golden/shade_ref.npz holds the shading of 2,000 seeded hits (and edge
cases: normals facing away from the light or the camera, sqr at and around
the shadow threshold 15) computed from src/mt_math/mt_vector_3d.c
(v3_sub, v3_scale, v3_normalize, v3_dot), compiled from the reference
sources. The oracle's restatement, which the kernels equal bit for bit on
every rendered pixel (tests/test_gpu_parity.py), must agree with it within the
RGB tolerance of the path: 1/255 per channel. v3_normalize multiplies by
1 / sqrt where the shader's normalize is restated as a division, so the two
differ by at most a few ulps; the test states that bound too."""
import os

import numpy as np

from conftest import GOLDEN

TOL_RGB = 1.0 / 255.0   # the path's RGB tolerance
TOL_FLOAT = 2.5e-7      # what the two normalizations differ by on these inputs


def test_shading_matches_reference_vector_helpers(oracle):
    g = dict(np.load(os.path.join(GOLDEN, "shade_ref.npz")))
    for shoot in (0, 1):
        mine = oracle.shade(g["isp"], g["nrm"], g["csv"], g["light"], g["sqr"], shoot, g["col"])
        ref = g[f"ref_shoot{shoot}"]
        err = np.abs(mine - ref).max()
        assert err <= TOL_FLOAT < TOL_RGB, (shoot, err)
        q = lambda a: np.clip(np.floor(a * 255.0 + 0.5), 0, 255)  # noqa: E731
        assert np.abs(q(mine) - q(ref)).max() <= 1

def test_shadow_threshold_of_both(oracle):
    """step(sqr, 15.0): sqr = 15 lights the hit, the next float above does
    not, in the oracle and in the reference-helper formula alike."""
    isp = np.array([[600.0, 100.0, 900.0]] * 2, np.float32)
    light = np.array([420.0, 200.0, 680.0], np.float32)
    nrm = (light - isp).astype(np.float32)  # facing the light
    csv = np.array([[0.0, -400.0, -700.0]] * 2, np.float32)
    col = np.array([[0.5, 0.6, 0.7, 1.0]] * 2, np.float32)
    sqr = np.array([15.0, np.nextafter(np.float32(15.0), np.float32(16.0))], np.float32)
    for reference in (False, True) if oracle.ref() is not None else (False,):
        out = oracle.shade(isp, nrm, csv, light, sqr, 0, col, reference=reference)
        assert (out[0, :3] > out[1, :3]).all(), (reference, out)
