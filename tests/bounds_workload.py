"""Workload run by tests/test_gpu_bounds.py in a child process, under
whichever build of libsph_cuda SPH_CUDA_LIB selects: a dam break with the
moving mover, hand-placed edge cases (a bucket over its cap, x == max_x,
coincident particles), a small ensemble, the learned step with its
fallback, the neighbour lists and a liquid image.  Prints one JSON line:
the bounds flags and a digest of every result."""
import ctypes
import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))

from make_golden import EDGE_CONFIG  # noqa: E402
from sph_gb300 import Ensemble, LearnedModel, Simulation, lib, scenes  # noqa: E402

digest = hashlib.sha256()


def add(*arrays):
    for a in arrays:
        digest.update(np.ascontiguousarray(a).tobytes())


sc = scenes.config2(16_384)
with Simulation.from_scene(sc) as s:
    s.step_schedule([sc.params_at(t).as_dict() for t in range(40)])
    st = s.download()
    add(st["x"], st["y"], st["v_x"], st["density"])
    counts, ids = s.neighbor_lists()
    add(counts, ids)
    add(s.render_liquid(320, 160))
    with LearnedModel(0, seed=5) as m:
        s.set_learned(m, 0.01)
        s.step(sc.params_at(40).as_dict(), 3)
        st = s.download()
        add(st["x"], st["y"])
        s.set_learned(None)

g = np.load(os.path.join(ROOT, "tests", "golden", "edges.npz"))
params = scenes.Params().as_dict()
with Simulation(params, EDGE_CONFIG, len(g["x"])) as s:
    s.upload(g["x"], g["y"])
    s.step(params, 5)
    st = s.download()
    add(st["x"], st["y"], st["density"])

scs = [scenes.ensemble_scene(9100 + k, f"e{k}", (400, 3000)) for k in range(4)]
e = Ensemble(scs)
e.upload_scenes()
e.step(None, 20)
st = e.download()
add(st["x"], st["y"])
e.close()

flags = ctypes.c_uint(0)
lib().sph_cuda_bounds_errors(ctypes.byref(flags))
print(json.dumps({"checked": int(lib().sph_cuda_bounds_checked()), "flags": int(flags.value),
                  "digest": digest.hexdigest()}))
