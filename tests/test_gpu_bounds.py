"""The bounds-checked build (-DSPH_BOUNDS_CHECK), the stand-in for a memory
checker: on a workload that covers the step, the edge cases, ensembles, the
learned step, the neighbour lists and the liquid image, no data-dependent
index may leave its array, and the results must equal the normal build's
bit for bit."""
import json
import os
import subprocess
import sys

import pytest

from sph_gb300 import build

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def run(lib_path):
    env = dict(os.environ, SPH_CUDA_LIB=lib_path)
    r = subprocess.run([sys.executable, os.path.join(HERE, "bounds_workload.py")], env=env,
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    return json.loads(r.stdout.strip().splitlines()[-1])


def test_checked_build_finds_no_bad_index(cuda_lib):
    checked = run(build.build_checked())
    normal = run(build.LIB)
    assert checked["checked"] == 1 and normal["checked"] == 0
    assert checked["flags"] == 0, checked
    assert checked["digest"] == normal["digest"]
