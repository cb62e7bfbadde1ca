import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300)")


def gpu_available() -> bool:
    try:
        import ctypes

        cudart = None
        for name in ("libcudart.so", "libcudart.so.13", "libcudart.so.12"):
            try:
                cudart = ctypes.CDLL(name)
                break
            except OSError:
                continue
        if cudart is None:
            return os.path.exists("/dev/nvidia0")
        n = ctypes.c_int(0)
        return cudart.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0
    except Exception:
        return False


@pytest.fixture(scope="session")
def golden():
    return np.load(os.path.join(GOLDEN, "golden.npz"))


@pytest.fixture(scope="session")
def dpca():
    """The product library, built if needed (loading fails loudly otherwise)."""
    from distpca_gb300 import build as B

    B.build()
    import distpca_gb300 as D

    D.lib()
    return D


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O

    O.build()
    return O


def fileset(name: str):
    from distpca_gb300 import synth

    prefix = os.path.join(GOLDEN, name)
    with open(prefix + ".fam") as f:
        n_ind = sum(1 for _ in f)
    with open(prefix + ".bim") as f:
        n_snp = sum(1 for _ in f)
    return prefix, n_ind, n_snp, synth.read_bed(prefix, n_ind, n_snp)


def run_flags(golden, run: str) -> dict:
    flags = list(golden[f"run_{run}_flags"])
    out = {}
    for i in range(0, len(flags), 2):
        key = flags[i].lstrip("-")
        val = flags[i + 1]
        out[key] = float(val) if key == "tol" else int(val)
    return out


def align_signs(u: np.ndarray, ref: np.ndarray) -> np.ndarray:
    s = np.sign(np.sum(u * ref, axis=0))
    s[s == 0] = 1
    return u * s
