"""Checkpoint and resume: a handle restored from a saved state continues
bit for bit as the saved handle does; mismatched or damaged files are
rejected."""
import numpy as np
import pytest

from conftest import bits_equal
from sph_gb300 import Ensemble, Simulation, SphError, scenes

pytestmark = pytest.mark.gpu

FIELDS = ("x", "y", "v_x", "v_y", "density", "density_near")


def test_resume_is_bit_exact(cuda_lib, tmp_path):
    sc = scenes.config2(16_384)
    sched = [sc.params_at(t).as_dict() for t in range(40)]
    path = tmp_path / "state.ckpt"
    with Simulation.from_scene(sc) as a:
        a.step_schedule(sched[:25])
        a.save_state(path)
        saved = a.download()
        a.step_schedule(sched[25:])
        ref = a.download()
        c_ref = a.counters()
    with Simulation(sc.params.as_dict(), sc.config(), sc.n) as b:
        b.load_state(path)
        assert all(bits_equal(b.download()[f], saved[f]) for f in FIELDS)
        b.step_schedule(sched[25:])
        got = b.download()
        for f in FIELDS:
            assert bits_equal(got[f], ref[f]), f
        assert b.counters()["steps"] == c_ref["steps"]


def test_ensemble_checkpoint_and_rejections(cuda_lib, tmp_path):
    scs = [scenes.ensemble_scene(9000 + s, f"s{s}", (500, 3000)) for s in range(3)]
    path = tmp_path / "ens.ckpt"
    e = Ensemble(scs)
    e2 = Ensemble(scs)
    try:
        e.upload_scenes()
        e.step(None, 12)
        e.save_state(path)
        e.step(None, 5)
        ref = e.download()
        e2.load_state(path)
        e2.step(None, 5)
        got = e2.download()
        assert all(bits_equal(got[f], ref[f]) for f in FIELDS)
    finally:
        e.close()
        e2.close()
    sc = scenes.config1()
    with Simulation(sc.params.as_dict(), sc.config(), sc.n) as s:
        with pytest.raises(SphError):
            s.load_state(path)  # three scenes into a one-scene handle
        bad = tmp_path / "bad.ckpt"
        bad.write_bytes(b"not a checkpoint")
        with pytest.raises(SphError):
            s.load_state(bad)
        with pytest.raises(SphError):
            s.load_state(tmp_path / "missing.ckpt")
