"""Synthetic scenes: sizes, fill fractions and seeds as documented."""
import math

import numpy as np

from sph_gb300 import scenes


def test_dam_break_4m_geometry():
    sc = scenes.config2()
    assert sc.n == 4_194_304 and sc.size_x == 3590 and sc.size_y == 1795
    assert sc.x.max() < 1196.1 and sc.y.max() < 876.6
    # fill fraction of config 1 kept (0.25 per particle)
    assert abs(sc.n * 0.25 / (3590 * 1795) - 3000 * 0.25 / (96 * 48)) < 1e-3
    cx, cy = sc.mover_at(60)
    assert cx == np.float32(598 + 20 * math.sin(2 * math.pi * 60 / 240)) and cy == np.float32(438)
    assert scenes.algorithmic_bytes_per_step(sc.n, sc.cells) == 1_009_074_464


def test_splitmix_deterministic():
    a = scenes.uniform(5, np.arange(10, dtype=np.uint64))
    b = scenes.uniform(5, np.arange(10, dtype=np.uint64))
    assert np.array_equal(a, b) and (a >= 0).all() and (a < 1).all()
    assert not np.array_equal(a, scenes.uniform(6, np.arange(10, dtype=np.uint64)))


def test_ensemble_scene_statistics():
    e = scenes.config3(nscenes=64)
    ns = np.array([s.n for s in e])
    assert ns.min() >= 1024 and ns.max() <= 65536
    for s in e:
        area = s.box[1] * s.box[3]
        f = s.n * 0.25 / area
        assert 0.19 < f < 0.51
        assert 1.0 <= s.box[1] / s.box[3] <= 4.0 + 1e-6
        assert 0.1 <= s.params.k <= 0.5 and 1.0 <= s.params.k_near <= 3.0 and 0 <= s.params.sigma <= 1
        assert s.x.min() > -0.02 and s.x.max() < s.box[1] and s.y.max() < s.box[3]
        assert s.size_x == math.ceil(s.box[1]) and s.size_y == math.ceil(s.box[3])
    again = scenes.config3(nscenes=3)
    assert all(np.array_equal(a.x, b.x) for a, b in zip(e[:3], again))
