import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")
GOLDEN_CASES = ["demtif", "fbm_slope", "fbm_hydro", "quantised"]


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the kernels through the C ABI")


def load_golden(name):
    with np.load(os.path.join(GOLDEN, name + ".npz")) as z:
        return {k: z[k] for k in z.files}


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    return oracle.Oracle()


@pytest.fixture(scope="session")
def ctx():
    """One pargo context for the GPU tests (fails loudly when the library or
    the GPU is missing -- there is no fallback to skip to)."""
    from pargo_gb300 import abi
    c = abi.Context(0)
    yield c
    c.close()


def bits_equal(a, b):
    a = np.ascontiguousarray(a, np.float64)
    b = np.ascontiguousarray(b, np.float64)
    return a.shape == b.shape and np.array_equal(a.view(np.int64), b.view(np.int64))


def near_zero_dem(rows, cols, seed):
    """Sea-level flats (0.0), tiny heights around the gap (0 .. 5e-3, which
    spans the binades where x + gap leaves x's binade or rounds on a tie) and
    a few negative cells, with pits in all of them."""
    rng = np.random.default_rng(seed)
    dem = rng.uniform(0.0, 5e-3, (rows, cols)).astype(np.float32)
    dem[:, : cols // 3] = 0.0
    dem[rows // 2:, cols // 3: cols // 2] = -rng.uniform(0.0, 2e-3, (rows - rows // 2, cols // 2 - cols // 3))
    pits = rng.random((rows, cols)) < 0.05
    dem[pits] = np.float32(0.0)
    dem[5:9, 5:9] = np.float32(2.0 ** -9)
    return dem
