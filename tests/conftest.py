"""Shared fixtures.

The reference's test set-up (tests/conftest.py of MikeSWang/Triumvirate):
box 1000 Mpc/h, 64^3 mesh, TSC, no interlacing, 4 linear bins 0.005-0.105
h/Mpc (Fourier) or 50-150 Mpc/h (configuration), a 3-particle data
catalogue and 30 000 uniform randoms drawn with seed 42.
"""
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = Path(__file__).resolve().parent / "golden"


def pytest_configure(config):
    config.addinivalue_line(
        "markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope='session')
def golden_dir():
    return GOLDEN


def load_golden(name):
    return np.loadtxt(GOLDEN / name, unpack=True)


@pytest.fixture(scope='session')
def data_catalogue_array():
    """x, y, z, nz of the 3-particle data catalogue."""
    return np.loadtxt(GOLDEN / "test_data_catalogue.txt")


@pytest.fixture(scope='session')
def rand_catalogue_array():
    """The reference's random catalogue (conftest.py:173-195 there)."""
    rng = np.random.default_rng(seed=42)
    x, y, z = rng.uniform(-500., 500., size=(3, 30000))
    return np.column_stack([x, y, z, np.full(30000, 3.e-9)])


BOX = 1000.
NMESH = 64
KBINS = (0.005, 0.105, 4)
RBINS = (50., 150., 4)

# (kind, degrees, form, idx_bin, golden file)
THREEPT_CASES = [
    ('bispec', (0, 0, 0), 'diag', None, 'bk000_diag_{}.txt'),
    ('bispec', (2, 0, 2), 'diag', None, 'bk202_diag_{}.txt'),
    ('bispec', (0, 0, 0), 'row', 0, 'bk000_row0_{}.txt'),
    ('3pcf', (0, 0, 0), 'diag', None, 'zeta000_diag_{}.txt'),
    ('3pcf', (2, 0, 2), 'diag', None, 'zeta202_diag_{}.txt'),
    ('3pcf', (0, 0, 0), 'row', 0, 'zeta000_row0_{}.txt'),
]
