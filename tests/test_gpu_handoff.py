"""Asynchronous coordinate hand-off: double-buffered packed coordinates
copied on their own stream must equal the synchronous packing of the same
states, and waiting is required and checked."""
import numpy as np
import pytest

from sph_gb300 import Simulation, SphError, scenes
from sph_gb300.simulation import PinnedArray

pytestmark = pytest.mark.gpu


def test_async_pack_equals_sync(cuda_lib):
    sc = scenes.config2(65_536)
    bufs = [PinnedArray((sc.n, 2), np.int16) for _ in range(2)]
    try:
        with Simulation.from_scene(sc) as a, Simulation.from_scene(sc) as b:
            for t in range(12):
                p = sc.params_at(t).as_dict()
                a.step(p)
                b.step(p)
                ref = a.pack_coords()
                b.pack_coords_async(bufs[t % 2].array)
                if t > 0:
                    b.wait_coords(bufs[(t - 1) % 2].array)
                    assert np.array_equal(bufs[(t - 1) % 2].array, prev)
                prev = ref
            b.wait_coords(bufs[11 % 2].array)
            assert np.array_equal(bufs[11 % 2].array, prev)
            with pytest.raises(SphError):
                b.wait_coords(bufs[0].array)  # nothing pending any more
    finally:
        for x in bufs:
            x.free()
