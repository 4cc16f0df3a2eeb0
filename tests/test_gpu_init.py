"""On-device scene initialisation: lattice blocks generated on the GPU must
equal, bit for bit, the host generator's scenes, and step identically."""
import numpy as np
import pytest

from conftest import bits_equal
from sph_gb300 import Ensemble, Simulation, SphError, scenes

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [3000, 65_536, 4_194_304])
def test_dam_break_on_device_equals_host(cuda_lib, n):
    sc = scenes.config1() if n == 3000 else scenes.config2(n)
    with Simulation(sc.params.as_dict(), sc.config(), sc.n) as dev:
        dev.init_lattice([sc.meta["lattice"]])
        st = dev.download()
        assert bits_equal(st["x"], sc.x) and bits_equal(st["y"], sc.y)
        assert not st["v_x"].any() and not st["v_y"].any()
        if n <= 65_536:
            with Simulation.from_scene(sc) as host:
                sched = [sc.params_at(t).as_dict() for t in range(6)]
                dev.step_schedule(sched)
                host.step_schedule(sched)
                a, b = dev.download(), host.download()
                for f in ("x", "y", "v_x", "v_y", "density"):
                    assert bits_equal(a[f], b[f]), f


def test_ensemble_and_piles_on_device(cuda_lib):
    for scs in (scenes.config3(8), scenes.config5(6)):
        e = Ensemble(scs)
        try:
            e.init_lattice([s.meta["lattice"] for s in scs])
            st = e.download()
            assert bits_equal(st["x"], np.concatenate([s.x for s in scs]))
            assert bits_equal(st["y"], np.concatenate([s.y for s in scs]))
            with pytest.raises(SphError):
                e.init_lattice([s.meta["lattice"] for s in scs[:-1]])
        finally:
            e.close()


def test_bad_blocks_rejected(cuda_lib):
    sc = scenes.config1()
    with Simulation(sc.params.as_dict(), sc.config(), sc.n) as s:
        bad = dict(sc.meta["lattice"], cols=0)
        with pytest.raises(SphError):
            s.init_lattice([bad])
        big = dict(sc.meta["lattice"], n=sc.n + 1)
        with pytest.raises(SphError):
            s.init_lattice([big])
