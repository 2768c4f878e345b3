import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")
S = 1800.0
LEVELS = 12
BASECUBE = (0.0, S, S, S)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs libqbcuda kernels)")


@pytest.fixture(scope="session")
def lib():
    import qubatron_gb300 as qb
    return qb.load()


@pytest.fixture(scope="session")
def oracle():
    from oracle import qbo
    qbo.build_oracle()
    qbo.qbo()
    return qbo


@pytest.fixture(scope="session")
def five_point():
    return dict(np.load(os.path.join(GOLDEN, "five_point.npz")))


@pytest.fixture(scope="session")
def floor50k():
    return dict(np.load(os.path.join(GOLDEN, "floor50k.npz")))


@pytest.fixture(scope="session")
def floor50k_scene(lib):
    from qubatron_gb300 import scenes
    return scenes.make_scene(scenes.scaled_spec("floor1m", 50_000))
