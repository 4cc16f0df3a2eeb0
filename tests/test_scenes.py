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


def test_skewed_scene_statistics():
    sc = scenes.config5(nscenes=48)
    ns = np.array([s.meta["n_total"] for s in sc])
    assert ns.min() >= 512 and ns.max() <= 32768
    occ = []
    for s in sc:
        m = s.meta
        assert s.n == m["n_pile"] and m["blob_x"].shape[0] == m["n_total"] - m["n_pile"]
        assert 0.49 <= m["n_pile"] / m["n_total"] <= 0.81
        assert 1 <= len(m["blobs"]) <= 6
        for b in m["blobs"]:
            assert b["sigma"] >= 3.0 or b["sigma"] >= s.box[1] / 4 - 1e-9
        x = np.concatenate([s.x, m["blob_x"]])
        y = np.concatenate([s.y, m["blob_y"]])
        assert x.min() >= 0 and x.max() < s.box[1] and y.min() >= 0 and y.max() < s.box[3]
        assert 1.0 <= s.box[1] / s.box[3] <= 2.0 + 1e-6
        k = np.floor(y).astype(np.int64) * s.size_x + np.floor(x).astype(np.int64)
        occ.append(np.bincount(k).max())
    # cell occupancies up to about a dozen per h^2 cell, far below the 100 cap
    assert 6 <= max(occ) <= 30
    again = scenes.config5(nscenes=2)
    assert all(np.array_equal(a.meta["blob_x"], b.meta["blob_x"]) for a, b in zip(sc[:2], again))


def test_learned_training_scenes():
    tr = scenes.learned_training_scenes(8, 65_536)
    assert all(s.n == 65_536 for s in tr)
    ks = [s.params.k for s in tr]
    assert len(set(ks)) == 8 and all(0.1 <= k <= 0.5 for k in ks)
    assert all(1.0 <= s.params.k_near <= 3.0 and 0.0 <= s.params.sigma <= 1.0 for s in tr)
    assert all(s.mover_period == 0.0 for s in tr)
    assert np.array_equal(tr[0].x, scenes.config2(65_536).x)
