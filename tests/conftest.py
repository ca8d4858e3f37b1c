import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")

# D2Q9 vectors (simuverse/src/fluid/mod.rs:22-52)
EX = np.array([0, 1, 0, -1, 0, 1, -1, -1, 1])
EY = np.array([0, 0, -1, 0, 1, -1, -1, 1, 1])


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA library")


@pytest.fixture(scope="session")
def native():
    """liblbm.so, built in-tree if needed (nvcc cross-compiles without a GPU)."""
    from simuverse_gb300 import build

    build.build()
    import simuverse_gb300

    return simuverse_gb300.load()


@pytest.fixture(scope="session")
def gpu(native):
    """The CUDA library on a real GPU; fails (does not skip) when no GPU is visible."""
    import torch

    if not torch.cuda.is_available():
        pytest.fail("no CUDA device visible for a gpu-marked test")
    return native


def comparable_slots(info):
    """Boolean (9, ny, nx) mask of the population slots a fluid cell can read.

    Excluded are wall-to-wall slots (slot k of a solid cell whose neighbour c+e_k is also
    solid): the reference's boundary dispatch races on them and no fluid cell reads them.
    """
    mat = info["material"]
    solid = (mat == 2) | (mat == 4)
    ny, nx = mat.shape
    keep = np.ones((9,) + mat.shape, bool)
    ys, xs = np.mgrid[0:ny, 0:nx]
    for k in range(9):
        px, py = xs + EX[k], ys + EY[k]
        inb = (px >= 0) & (px < nx) & (py >= 0) & (py < ny)
        nb_solid = np.zeros_like(solid)
        nb_solid[inb] = solid[py[inb], px[inb]]
        keep[k] &= ~(solid & nb_solid)
    return keep


def max_rel_err(a, b, floor):
    return float(np.max(np.abs(a.astype(np.float64) - b.astype(np.float64)) / np.maximum(np.abs(b), floor)))


def rel_l2(a, b):
    a = a.astype(np.float64)
    b = b.astype(np.float64)
    den = np.sqrt(np.sum(b * b))
    return float(np.sqrt(np.sum((a - b) ** 2)) / (den if den > 0 else 1.0))
