import importlib.util
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "3d-fluid-numerical-simulation-software_gb300")
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (PKG, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN_CASES = ["duct_9x9x17", "duct_9x9x17_sw_nnd", "duct_9x9x17_laminar_cons", "duct_9x9x17_muscl2u_global",
                "rotor_9x9x33", "rotor_9x9x33_mg"]
# fixtures the GPU parity tests check against the reference's own outputs only: Spalart-Allmaras (not restated by the
# CPU oracle) and JST (restated by the oracle, which test_oracle_golden checks against the same fixtures)
REFERENCE_ONLY_CASES = ["duct_9x9x17_jst", "rotor_9x9x33_jst_mg", "duct_9x9x17_sa", "rotor_9x9x33_sa"]


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and the built libgbturbo.so")


def load_golden(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    return {k: z[k] for k in z.files}


def golden_dir(name):
    return os.path.join(GOLDEN, name)


def rel_err(a, b, floor=1e-6):
    """Normwise relative error per trailing component, max over components. A component whose
    norm is below `floor` times the largest component's norm (rounding noise of a quantity that
    is zero in exact arithmetic) is measured against that floor instead of its own norm."""
    a = np.asarray(a, dtype=np.float64)
    a = a.reshape(-1, a.shape[-1]) if a.ndim > 1 else a.reshape(-1, 1)
    b = np.asarray(b, dtype=np.float64).reshape(a.shape)
    num = np.linalg.norm(a - b, axis=0)
    den = np.linalg.norm(b, axis=0)
    den = np.maximum(den, floor * max(float(den.max()), 1e-300))
    return float(np.max(num / den))


@pytest.fixture(scope="session")
def meshgen():
    import meshgen as mg
    return mg


@pytest.fixture(scope="session")
def oracle_mod():
    import pyoracle
    pyoracle.build()
    return pyoracle


@pytest.fixture(scope="session")
def gbturbo():
    import gbturbo as g
    return g


@pytest.fixture(scope="session")
def gpu_lib():
    """the built GPU library; on a GPU machine a missing library is a failure, not a skip"""
    import build as pkg_build
    pkg_build.build()
    import gbturbo as g
    g.load()
    return g
