"""CPU restatement of the render rank's liquid image -- TEST INFRASTRUCTURE
ONLY (the checker of sph_render_liquid; nothing in the product imports it).

The reference draws the liquid with OpenGL (liquid_gl.c:305-447), which
cannot run here; this is its arithmetic, restated from the sources:

* splat: point sprites of diameter 0.020 x screen width (renderer.c:224)
  divided by the texture reduction 2 (liquid_gl.c:47, 77), centred at the
  window position of the point (short / SHRT_MAX, renderer.c:333-337);
  per pixel r^2 = |2 gl_PointCoord - 1|^2, discarded above 0.34, intensity
  1 - 3 r^2 (shaders/liquid_particle.frag:10-20), blended additively into
  an 8-bit texture (liquid_gl.c:106, 318-343): sum of round(255 i),
  saturated at 255;
* blur: 15 taps at 0, +-0.004 k texture units along y then x
  (shaders/vert_blur.vert:12-26, shaders/horz_blur.vert), weights of
  shaders/blur.frag:12-29, bilinear and clamped to the edge
  (liquid_gl.c:107-110), stored back to 8 bits after each pass;
* composite: bilinear sample at screen resolution, discard below 0.1,
  colour (w, w, 1), w = smoothstep(-0.15, -0.1, -a), alpha
  0.75 smoothstep(0.1, 0.11, a) (shaders/render_liquid_texture.frag:11-17)
  over black (liquid_gl.c:436-444).

Arithmetic is float32 in the kernels' order; images bottom row first until
the final RGB (top row first)."""
from __future__ import annotations

import numpy as np

# The reference's constants, by source (tests/golden/liquid_shaders.json
# holds them as read out of those sources, and the tests compare the two).
TAPS = np.array([0.159576912161, 0.147308056121, 0.115876621105, 0.0776744219933,
                 0.0443683338718, 0.0215963866053, 0.00895781211794, 0.0044299121055113265],
                np.float32)            # blur.frag:12-29: centre, then taps +-1 .. +-7
BLUR_STEP = 0.004                      # vert_blur.vert / horz_blur.vert:13-26: texture units per tap
SPRITE_DIAMETER = 0.020                # renderer.c:224: sprite diameter / screen width
REDUCTION = 2                          # liquid_gl.c:44-48: texture size = screen / 2
DISCARD_R2 = 0.34                      # liquid_particle.frag:14: discard r^2 above this
INTENSITY = (1.0, 3.0)                 # liquid_particle.frag:19: 1.0 - 3.0 r^2
COMPOSITE_DISCARD = 0.1                # render_liquid_texture.frag:11: discard alpha below
ALPHA_EDGES = (0.1, 0.11)              # render_liquid_texture.frag:14: smoothstep of alpha
WHITE_EDGES = (-0.15, -0.1)            # render_liquid_texture.frag:15: smoothstep of -alpha
ALPHA_SCALE = 0.75                     # render_liquid_texture.frag:17: output alpha scale
F = np.float32


def splat(coords: np.ndarray, width: int, height: int) -> np.ndarray:
    w, h = width // REDUCTION, height // REDUCTION
    radius = F(0.5) * (F(width) * F(SPRITE_DIAMETER) / F(REDUCTION))
    inv = F(1.0) / radius
    acc = np.zeros((h, w), np.int64)
    reach = F(0.5831) * radius + F(1.0)
    for cxs, cys in coords.astype(np.int64):
        px, py = F(cxs) / F(32767.0), F(cys) / F(32767.0)
        cx = (px + F(1.0)) * F(0.5) * F(w)
        cy = (py + F(1.0)) * F(0.5) * F(h)
        x0, x1 = max(0, int(np.floor(cx - reach))), min(w - 1, int(np.ceil(cx + reach)))
        y0, y1 = max(0, int(np.floor(cy - reach))), min(h - 1, int(np.ceil(cy + reach)))
        if x1 < x0 or y1 < y0:
            continue
        xs = np.arange(x0, x1 + 1)
        ys = np.arange(y0, y1 + 1)
        dx = (xs.astype(np.float32) + F(0.5) - cx) * inv
        dy = (ys.astype(np.float32) + F(0.5) - cy) * inv
        r2 = dy[:, None] * dy[:, None] + dx[None, :] * dx[None, :]
        v = np.rint((F(INTENSITY[0]) - F(INTENSITY[1]) * r2) * F(255.0)).astype(np.int64)
        v[(r2 > F(DISCARD_R2)) | (v < 0)] = 0
        acc[y0:y1 + 1, x0:x1 + 1] += v
    return np.minimum(acc, 255).astype(np.uint8)


def _lerp(line: np.ndarray, t: np.ndarray) -> np.ndarray:
    n = line.shape[-1]
    f = np.floor(t)
    a = (t - f).astype(np.float32)
    i0 = f.astype(np.int64)
    j0 = np.clip(i0, 0, n - 1)
    j1 = np.clip(i0 + 1, 0, n - 1)
    lv = line.astype(np.float32)
    return (F(1.0) - a) * lv[..., j0] + a * lv[..., j1]


def blur(tex: np.ndarray, vertical: bool) -> np.ndarray:
    img = tex.T if vertical else tex  # lines along the blurred axis
    length = img.shape[1]
    pos = np.arange(length, dtype=np.float32)
    s = TAPS[0] * img.astype(np.float32)
    for k in range(1, 8):
        o = F(BLUR_STEP) * F(k) * F(length)
        s = s + TAPS[k] * (_lerp(img, pos - o) + _lerp(img, pos + o))
    out = np.clip(np.rint(s), 0, 255).astype(np.uint8)
    return out.T if vertical else out


def _smoothstep(e0, e1, x):
    t = np.clip((x - F(e0)) / (F(e1) - F(e0)), 0.0, 1.0).astype(np.float32)
    return t * t * (F(3.0) - F(2.0) * t)


def composite(a: np.ndarray, width: int, height: int) -> np.ndarray:
    h, w = a.shape
    X = np.arange(width, dtype=np.float32)
    Y = np.arange(height, dtype=np.float32)
    u = (X + F(0.5)) / F(width) * F(w) - F(0.5)
    v = (Y + F(0.5)) / F(height) * F(h) - F(0.5)
    fu, fv = np.floor(u), np.floor(v)
    au, av = (u - fu).astype(np.float32), (v - fv).astype(np.float32)
    ia = np.clip(fu.astype(np.int64), 0, w - 1)
    ib = np.clip(fu.astype(np.int64) + 1, 0, w - 1)
    ja = np.clip(fv.astype(np.int64), 0, h - 1)
    jb = np.clip(fv.astype(np.int64) + 1, 0, h - 1)
    af = a.astype(np.float32)
    s00, s01 = af[ja][:, ia], af[ja][:, ib]
    s10, s11 = af[jb][:, ia], af[jb][:, ib]
    au2, av2 = au[None, :], av[:, None]
    alpha = ((F(1.0) - av2) * ((F(1.0) - au2) * s00 + au2 * s01) +
             av2 * ((F(1.0) - au2) * s10 + au2 * s11)) / F(255.0)
    o = F(ALPHA_SCALE) * _smoothstep(ALPHA_EDGES[0], ALPHA_EDGES[1], alpha)
    white = _smoothstep(WHITE_EDGES[0], WHITE_EDGES[1], -alpha)
    keep = alpha >= F(COMPOSITE_DISCARD)
    r = np.where(keep, white * o, F(0.0))
    b = np.where(keep, o, F(0.0))
    rgb = np.stack([r, r, b], axis=-1)
    out = np.rint(rgb * F(255.0)).astype(np.uint8)
    return out[::-1]  # top row first


def render(coords: np.ndarray, width: int, height: int):
    """(rgb top row first, blurred alpha bottom row first, splat alpha)."""
    a0 = splat(coords, width, height)
    a2 = blur(blur(a0, True), False)
    return composite(a2, width, height), a2, a0
