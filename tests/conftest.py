"""Shared test setup: import paths, the `gpu` marker, oracle and fixtures."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, os.path.join(ROOT, "speckle-stacker_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libsmip_gpu.so")


def golden(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


@pytest.fixture(scope="session")
def oracle():
    from oracle import Oracle, build

    lib = os.path.join(ROOT, "oracle", "_build", "libsmip_oracle.so")
    if not os.path.exists(lib):
        build(reference="/nonexistent")
    return Oracle()


@pytest.fixture(scope="session")
def smip():
    import smip_gb300

    smip_gb300._L()  # fails loudly when the library is not built
    return smip_gb300


def rel_l2(a, b):
    a = np.asarray(a, np.complex128).ravel()
    b = np.asarray(b, np.complex128).ravel()
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def phase_err(ph, ref, mask):
    return np.abs(np.angle(ph[mask] * np.conj(ref[mask])))
