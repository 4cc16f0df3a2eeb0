"""The C compute-rank program (sph_gb300/host/compute_rank.c): the
reference's start_simulation loop on libsph_cuda with a stand-in render rank
that moves the mover and switches fluid presets between frames.  Its frames
must equal, bit for bit, the same run replayed through the Python binding
from its recorded initial state and per-step tunables."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from sph_gb300 import Simulation, _lib, build

pytestmark = pytest.mark.gpu


def run_compute_rank(tmp_path, n, steps, spf, preset_frames):
    build.build()
    prefix = str(tmp_path / "rank")
    r = subprocess.run([build.COMPUTE_RANK, str(n), str(steps), str(spf), prefix, "1920", "1080",
                        str(preset_frames)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    init = np.fromfile(prefix + ".init", np.float32).reshape(-1, 2)
    raw = open(prefix + ".tunables", "rb").read()
    sz = ctypes.sizeof(_lib.TunableParameters)
    tps = [_lib.TunableParameters.from_buffer_copy(raw[i:i + sz]) for i in range(0, len(raw), sz)]
    fr = open(prefix + ".frames", "rb").read()
    n_, nframes = np.frombuffer(fr[:8], np.int32)
    max_x, max_y, h = np.frombuffer(fr[8:20], np.float32)
    size_x, size_y = np.frombuffer(fr[20:28], np.uint32)
    frames = np.frombuffer(fr[28:], np.int16).reshape(int(nframes), int(n_), 2)
    return r.stdout, init, tps, frames, (float(max_x), float(max_y), float(h), int(size_x), int(size_y))


def as_dict(tp):
    return {name: getattr(tp, name) for name, _ in _lib.TunableParameters._fields_}


def test_compute_rank_matches_the_binding(cuda_lib, tmp_path):
    out, init, tps, frames, (max_x, max_y, h, sx, sy) = run_compute_rank(tmp_path, 1500, 160, 4, 8)
    n = init.shape[0]
    assert "frames 40" in out and len(tps) == 160 and frames.shape == (40, n, 2)
    # presets changed the fluid during the run and the mover moved
    assert len({(t.k, t.k_spring) for t in tps}) >= 3
    assert len({t.mover_center_x for t in tps}) > 30
    config = dict(box=(0.0, max_x, 0.0, max_y), spacing=h, size_x=sx, size_y=sy, max_bucket=100,
                  max_neighbors=400)
    with Simulation(as_dict(tps[0]), config, n) as s:
        s.upload(init[:, 0].copy(), init[:, 1].copy())
        f = 0
        for t, tp in enumerate(tps):
            s.step(as_dict(tp))
            if t % 4 == 3:
                assert np.array_equal(s.pack_coords(), frames[f]), f
                f += 1
        assert f == 40
