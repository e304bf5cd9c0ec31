"""Shared test set-up: import paths, the `gpu` marker and small synthetic cases."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "epspectral.jl_gb300")
for p in (ROOT, PKG, os.path.dirname(os.path.abspath(__file__))):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); parity tests of the library")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def holstein():
    """The 1D Holstein fixture of test/test_scgd0_holstein.jl:5-12 (t = 1, ω0 = 0.2, g2 = 0.2,
    nk = 64, T = 0.1, ωs = -4:0.02:4)."""
    from epspectral_gb300 import FrequencyGrid, synthetic
    ws = FrequencyGrid.from_nodes(np.arange(-200, 201) * 0.02)
    return dict(nk=64, t=1.0, w0=0.2, g2=0.2, T=0.1, ws=ws,
                setup=synthetic.holstein_1d_setup(64, 1.0, 0.2, 0.2, ws))
