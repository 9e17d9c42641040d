"""pytest configuration: the `gpu` marker and shared fixtures.

Tests marked `gpu` need a GB300 and the built library; everything else runs
on a CPU-only machine.
"""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden", "o3_reference_golden.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GPU and the built CUDA library")


@pytest.fixture(scope="session")
def golden():
    return dict(np.load(GOLDEN))


@pytest.fixture(scope="session")
def small_params():
    """The reference's O3 small-system test parameters without B-field
    (test/parameters/O3_no_bfield_small_system.in.xml)."""
    from oracle.dqmc_ref import Params
    return Params(L=4, slices=10, delta_tau=0.1, safe_mult=10, lambda_=0.5, r=2.0, c=3.0, u=1.0,
                  mu1=-0.5, mu2=-0.5, hoppings=(1.0, 0.5, -0.5, -1.0))
