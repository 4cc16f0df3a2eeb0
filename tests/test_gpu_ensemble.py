"""The batched ensemble: many scenes advanced by one set of launches per step.
Each scene must follow, bit for bit, the trajectory it has when run alone,
and the autotuned launch shapes must not change any result."""
import numpy as np
import pytest

import oracle
from conftest import bits_equal
from sph_gb300 import Ensemble, Simulation, scenes

pytestmark = pytest.mark.gpu

STEPS = 40


def small_scenes(k=6):
    return [scenes.ensemble_scene(7000 + s, f"small_{s}", (300, 4000)) for s in range(k)]


def run_alone(sc, steps):
    with Simulation.from_scene(sc) as s:
        s.step(sc.params.as_dict(), steps)
        return s.download(), s.diagnostics()


def run_ensemble(scs, steps, shapes=None, autotune=False, long_masks=False):
    e = Ensemble(scs)
    e.upload_scenes()
    if shapes is not None:
        e.set_launch_shapes(shapes)
    if long_masks:
        e.set_long_row_masks(True)
    if autotune:
        chosen = e.autotune(1)  # advances 48 steps
        # re-upload so every run starts from the same state
        e.upload_scenes()
        assert chosen == e.launch_shapes()
    e.step(None, steps)
    out = e.download(), e.scene_diagnostics()
    e.close()
    return out


def test_each_scene_matches_its_solo_run(cuda_lib):
    scs = small_scenes()
    st, diag = run_ensemble(scs, STEPS)
    off = np.concatenate([[0], np.cumsum([s.n for s in scs])])
    for k, sc in enumerate(scs):
        alone, d1 = run_alone(sc, STEPS)
        sl = slice(off[k], off[k + 1])
        for f in ("x", "y", "v_x", "v_y", "density", "density_near"):
            assert bits_equal(st[f][sl], alone[f]), (k, f)
        # same sums in another reduction order: equal to rounding
        assert np.allclose(diag[k], d1, rtol=1e-12, atol=0), k


def test_launch_shapes_do_not_change_results(cuda_lib):
    scs = small_scenes(4)
    ref, _ = run_ensemble(scs, 10)
    for shapes in ([128, 0, 512, 0, 128, 0], [256, 2, 256, 4, 256, 2], [512, 1, 128, 8, 64, 0]):
        got, _ = run_ensemble(scs, 10, shapes=shapes)
        for f in ref:
            assert bits_equal(got[f], ref[f]), (shapes, f)
    got, _ = run_ensemble(scs, 10, autotune=True)
    for f in ref:
        assert bits_equal(got[f], ref[f]), f


def test_long_row_masks_do_not_change_results(cuda_lib):
    """Dense scenes (cells of ~25 particles: stencil rows of ~75
    candidates) with and without long-row hit masks: the same bits."""
    scs = [scenes.dam_break(6400, 80, 64.0, 64.0, seed=90 + s, name=f"dense_{s}", lattice=0.2,
                            x0=0.1, y0=0.1) for s in range(3)]
    ref, rd = run_ensemble(scs, 8)
    got, gd = run_ensemble(scs, 8, long_masks=True)
    for f in ref:
        assert bits_equal(got[f], ref[f]), f
    assert np.array_equal(rd, gd)


def test_ensemble_scenes_follow_cpu_jacobi(cuda_lib):
    scs = small_scenes(3)
    st, _ = run_ensemble(scs, 3)
    off = np.concatenate([[0], np.cumsum([s.n for s in scs])])
    for k, sc in enumerate(scs):
        orc = oracle.Sim("port", sc.x, sc.y, sc.vx, sc.vy, sc.params.as_dict(), sc.config())
        orc.step(3, jacobi=True)
        b = orc.get()
        sl = slice(off[k], off[k + 1])
        for f in ("x", "y"):
            assert np.abs(st[f][sl] - b[f]).max() < 1e-4, (k, f)


def test_ensemble_rejects_per_step_tunables_and_wrong_counts(cuda_lib):
    from sph_gb300 import SphError
    scs = small_scenes(2)
    e = Ensemble(scs)
    with pytest.raises(SphError):
        e.upload(scs[0].x, scs[0].y)  # only one scene's particles
    e.upload_scenes()
    with pytest.raises(ValueError):
        e.step(scs[0].params.as_dict())
    e.set_scene_params(1, dict(scs[1].params.as_dict(), g=0.0))
    e.step(None, 2)
    e.close()
