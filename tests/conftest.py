import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

DATA_DIR = ROOT / "mocassin_xray_gb300" / "data"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels through libmcx.so)")


@pytest.fixture(scope="session")
def data_dir() -> Path:
    return DATA_DIR


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def decks(tmp_path_factory):
    """Small decks of the measured workloads, written once per session."""
    from mocassin_xray_gb300 import configs
    root = tmp_path_factory.mktemp("decks")
    return {
        "h_small": configs.h_sphere(root / "h_small", n=9, packets=20000, edge=6.0e18),
        "h_sphere": configs.h_sphere(root / "h_sphere"),
        "lognormal_small": configs.lognormal_gas(root / "ln_small", n=13, packets=20000, half_width=1.5e19),
        "xray_small": configs.xray_gas(root / "xr_small", n=11, packets=20000),
    }


def synthetic_recpdf(nu: np.ndarray, n_cells: int, seed: int = 0) -> np.ndarray:
    """A per-cell re-emission CDF with a recombination-like shape (test input
    for the transport before the emission phase runs)."""
    rng = np.random.default_rng(seed)
    C1 = n_cells + 1
    out = np.zeros((nu.size, C1), dtype=np.float32)
    for c in range(1, C1):
        kT = 0.1 + 0.4 * rng.random()
        w = np.where(nu >= 1.0, nu ** 3 * np.exp(-(nu - 1.0) / kT), 1e-3 * nu ** 0.5)
        cdf = np.cumsum(w)
        cdf /= cdf[-1]
        cdf[-1] = 1.0
        out[:, c] = cdf
    return out


def gpu_available() -> bool:
    try:
        import ctypes
        lib = ctypes.CDLL("libcuda.so.1")
        n = ctypes.c_int()
        return lib.cuInit(0) == 0 and lib.cuDeviceGetCount(ctypes.byref(n)) == 0 and n.value > 0
    except OSError:
        return False
