import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")
if GOLDEN not in sys.path:
    sys.path.insert(0, GOLDEN)

from make_golden import EDGE_CONFIG  # noqa: E402,F401  (grid of the hand-placed fixtures)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _built_oracle():
    """The CPU oracle is plain C; build it (and the reference, where its
    sources exist) once per session if missing."""
    import oracle
    if not os.path.exists(oracle.PORT_LIB) or (os.path.isdir(oracle.REF_SRC) and not oracle.ref_available()):
        oracle.build()
    subprocess.run(["make", "-s", "-C", oracle.HERE, "all"], check=True)
    yield


@pytest.fixture(scope="session")
def cuda_lib():
    """libsph_cuda, built if needed (nvcc cross-compiles without a GPU)."""
    from sph_gb300 import build
    build.build()
    from sph_gb300 import _lib
    return _lib.lib()


def golden(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def bits_equal(a, b):
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    return a.shape == b.shape and np.array_equal(a.view(np.int32), b.view(np.int32))


def rel_ok(a, b, rtol=1e-5):
    """Per element |a - b| <= rtol |b| with no absolute floor: where the
    reference value is exactly zero (a particle with no neighbour) the result
    must be an exact zero.  Returns (ok, largest relative error)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    if a.shape != b.shape:
        return False, float("inf")
    err = np.abs(a - b)
    nz = b != 0
    rel = np.where(nz, err / np.where(nz, np.abs(b), 1.0), np.where(err == 0, 0.0, np.inf))
    return bool(np.all(rel <= rtol)), float(rel.max(initial=0.0))
