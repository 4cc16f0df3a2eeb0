"""Headless liquid image on the GPU against its CPU restatement
(oracle/liquid_image.py): the splat is integer-exact, the blurred alpha
within one 8-bit level, the composite equal wherever the alpha is."""
import numpy as np
import pytest

from oracle import liquid_image as li
from sph_gb300 import Simulation, render_liquid, scenes, write_ppm

pytestmark = pytest.mark.gpu


def compare(coords, W, H):
    rgb, a2 = render_liquid(coords, W, H)
    ref_rgb, ref_a2, _ = li.render(coords, W, H)
    d = np.abs(a2.astype(int) - ref_a2.astype(int))
    assert d.max() <= 1 and (d == 0).mean() > 0.995, (d.max(), (d == 0).mean())
    e = np.abs(rgb.astype(int) - ref_rgb.astype(int)).max(axis=-1)
    assert (e <= 2).mean() > 0.99
    return rgb


def test_image_of_a_dam_break(cuda_lib, tmp_path):
    sc = scenes.config1()
    with Simulation.from_scene(sc) as s:
        s.step(sc.params.as_dict(), 60)
        coords = s.pack_coords()
        W, H = 640, 320
        rgb = compare(coords, W, H)
        rgb2 = s.render_liquid(W, H)
        assert np.array_equal(rgb, rgb2)  # from the handle, packed on the device
    assert (rgb[..., 2] > 0).mean() > 0.05  # the fluid is drawn
    write_ppm(str(tmp_path / "dam.ppm"), rgb)
    assert (tmp_path / "dam.ppm").stat().st_size == 15 + W * H * 3


def test_image_edges_and_crowding(cuda_lib):
    rng = np.random.default_rng(3)
    pts = np.concatenate([rng.integers(-32767, 32768, (300, 2)),
                          np.zeros((50, 2), np.int64),                      # crowded centre
                          [[-32767, -32767], [32767, 32767], [32767, -32767]]]).astype(np.int16)
    compare(pts, 500, 300)
    rgb, a = render_liquid(np.zeros((0, 2), np.int16), 64, 32)
    assert rgb.max() == 0 and a.max() == 0
