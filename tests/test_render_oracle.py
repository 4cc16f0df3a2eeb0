"""The CPU restatement of the liquid image (oracle/liquid_image.py): sanity
of each pass on hand-made inputs (no GPU)."""
import numpy as np

from oracle import liquid_image as li


def test_single_sprite_is_a_disc():
    W, H = 1000, 500
    a = li.splat(np.array([[0, 0]], np.int16), W, H)  # centre of the screen
    r = 0.5 * (W * 0.020 / 2)  # 5 pixel sprite radius at 1000 wide
    ys, xs = np.nonzero(a)
    cy, cx = (H // 2) / 2.0, (W // 2) / 2.0
    d2 = ((xs + 0.5 - cx) / r) ** 2 + ((ys + 0.5 - cy) / r) ** 2
    assert len(xs) > 0 and d2.max() <= 0.34 + 1e-6
    assert a.max() <= 255 and a[ys, xs].min() > 0


def test_additive_blend_saturates():
    W, H = 400, 200
    pts = np.zeros((40, 2), np.int16)  # 40 sprites on one spot
    a = li.splat(pts, W, H)
    assert a.max() == 255


def test_blur_conserves_mass_and_is_symmetric():
    t = np.zeros((64, 128), np.uint8)
    t[32, 64] = 200
    b = li.blur(t, False)
    assert abs(int(b.sum()) - 200) <= 8  # 8-bit rounding of 15 taps
    assert np.array_equal(b[32, 64 - 10:64], b[32, 65:75][::-1])
    assert li.TAPS[0] + 2 * li.TAPS[1:].sum() > 0.99


def test_composite_threshold():
    a = np.full((10, 20), 20, np.uint8)  # 0.078 < 0.1: discarded
    assert li.composite(a, 40, 20).max() == 0
    a[:] = 200  # 0.78: opaque blue-ish, no white
    rgb = li.composite(a, 40, 20)
    assert (rgb[..., 2] == 191).all() and (rgb[..., 0] == 0).all()
