import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "calypso-gap_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")
GOLDEN_MODEL = os.path.join(GOLDEN, "gap_parameters_c_diamond")
GOLDEN_FRAMES = os.path.join(GOLDEN, "ase_traj_frames.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def frames():
    return dict(np.load(GOLDEN_FRAMES))


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def golden_oracle_model(oracle_mod):
    return oracle_mod.Model(GOLDEN_MODEL)


@pytest.fixture(scope="session")
def gapgb_mod():
    import gapgb
    gapgb.build.build()
    gapgb.load()
    return gapgb
