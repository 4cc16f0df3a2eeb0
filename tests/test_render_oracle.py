"""The CPU restatement of the liquid image (oracle/liquid_image.py): sanity
of each pass on hand-made inputs (no GPU)."""
import numpy as np
import pytest

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


def _fixture():
    import json
    import os
    with open(os.path.join(os.path.dirname(__file__), "golden", "liquid_shaders.json")) as f:
        return json.load(f)


def test_restatement_uses_the_reference_shader_constants():
    """Every constant of the restatement equals the one read out of the
    reference's shaders and render code (tests/golden/liquid_shaders.json,
    written by tests/golden/make_shader_constants.py)."""
    c = _fixture()
    w = np.array(c["blur_weights_in_tap_order"], np.float32)
    assert c["blur_tap_order"][7] == "centre" and len(w) == 15
    assert np.array_equal(w[7], li.TAPS[0])
    assert np.array_equal(w[8:], li.TAPS[1:]) and np.array_equal(w[:7][::-1], li.TAPS[1:])
    steps = np.concatenate([np.arange(-7, 0), np.arange(1, 8)]) * li.BLUR_STEP
    for k in ("vertical_offsets", "horizontal_offsets"):
        assert np.allclose(c[k], steps, rtol=0, atol=1e-12), k
    for k in ("vertical_cross_offsets", "horizontal_cross_offsets"):
        assert not np.any(c[k]), k
    assert c["sprite_discard_r2"] == li.DISCARD_R2
    assert tuple(c["sprite_intensity"]) == li.INTENSITY
    assert c["composite_discard_alpha"] == li.COMPOSITE_DISCARD
    assert tuple(c["composite_alpha_edges"]) == li.ALPHA_EDGES
    assert tuple(c["composite_white_edges"]) == li.WHITE_EDGES
    assert c["composite_alpha_scale"] == li.ALPHA_SCALE
    assert c["sprite_diameter_per_screen_width"] == li.SPRITE_DIAMETER
    assert c["texture_reduction"] == li.REDUCTION


def test_shader_fixture_matches_the_reference_sources():
    """Where the reference checkout is present, its sources still give the
    committed fixture."""
    import os
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
    import make_shader_constants as m
    root = m.default_reference_root()
    if not os.path.isdir(os.path.join(root, "shaders")):
        pytest.skip("reference sources not present on this machine")
    assert m.read_constants(root) == _fixture()
