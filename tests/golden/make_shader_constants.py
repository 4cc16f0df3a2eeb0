"""Reads the constants of the reference's liquid rendering out of its own
sources and writes them to tests/golden/liquid_shaders.json, the fixture that
pins the CPU restatement of the liquid image (oracle/liquid_image.py) and,
through it, the CUDA kernels of sph_render_liquid.

Sources read (paths within the reference checkout):
  shaders/blur.frag:12-29             the 15 Gaussian weights, in tap order
  shaders/vert_blur.vert:13-26        the vertical taps' texture offsets
  shaders/horz_blur.vert:13-26        the horizontal taps' texture offsets
  shaders/liquid_particle.frag:10-20  the discard radius^2 and 1 - 3 r^2
  shaders/render_liquid_texture.frag:11-17  discard level, smoothstep edges,
                                      the 0.75 alpha scale
  src/renderer.c:224                  liquid sprite diameter / screen width
  src/liquid_gl.c:44-48               texture reduction (non-Raspberry-Pi)

Run from the repository root, where the reference checkout is reachable:
  python tests/golden/make_shader_constants.py [REFERENCE_ROOT]
(default: $SPH_REF_SRC/.. or a checkout named "reference" beside this
repository).  tests/test_render_oracle.py re-reads the sources the same way
wherever they exist and compares them with the committed fixture.
"""
from __future__ import annotations

import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "liquid_shaders.json")
NUM = r"[-+]?[0-9]*\.?[0-9]+(?:[eE][-+]?[0-9]+)?"


def default_reference_root() -> str:
    src = os.environ.get("SPH_REF_SRC")
    if src:
        return os.path.dirname(os.path.abspath(src))
    return os.path.join(os.path.dirname(os.path.dirname(os.path.dirname(HERE))), "reference")


def _read(root, rel):
    with open(os.path.join(root, rel)) as f:
        return f.read()


def _one(pattern, text, what):
    m = re.findall(pattern, text)
    if len(m) != 1:
        raise ValueError(f"{what}: expected one match of {pattern!r}, found {len(m)}")
    return m[0]


def read_constants(root: str) -> dict:
    blur = _read(root, "shaders/blur.frag")
    taps = re.findall(r"texture\(tex,\s*(blur_tex_coords\[\s*(\d+)\]|frag_tex_coord)\s*\)\.a\s*\*\s*(" + NUM + r")", blur)
    if len(taps) != 15:
        raise ValueError(f"blur.frag: expected 15 taps, found {len(taps)}")
    weights = [float(w) for _, _, w in taps]
    order = [("centre" if idx == "" else int(idx)) for _, idx, _ in taps]

    def offsets(name, comp):
        text = _read(root, f"shaders/{name}")
        found = re.findall(r"blur_tex_coords\[\s*(\d+)\]\s*=\s*frag_tex_coord\s*\+\s*mult\s*\*\s*vec2\(\s*("
                           + NUM + r")\s*,\s*(" + NUM + r")\s*\)", text)
        if len(found) != 14:
            raise ValueError(f"{name}: expected 14 offsets, found {len(found)}")
        mult = float(_one(r"float\s+mult\s*=\s*(" + NUM + r")\s*;", text, name))
        return [mult * float(v[1 + comp]) for v in sorted(found, key=lambda v: int(v[0]))], \
            [mult * float(v[2 - comp]) for v in sorted(found, key=lambda v: int(v[0]))]

    v_along, v_across = offsets("vert_blur.vert", 1)
    h_along, h_across = offsets("horz_blur.vert", 0)
    part = _read(root, "shaders/liquid_particle.frag")
    discard_r2 = float(_one(r"if\s*\(\s*rad_squared\s*>\s*(" + NUM + r")\s*\)", part, "liquid_particle.frag"))
    i0, i1 = _one(r"intensity\s*=\s*(" + NUM + r")\s*-\s*(" + NUM + r")\s*\*\s*rad_squared", part,
                  "liquid_particle.frag")
    comp = _read(root, "shaders/render_liquid_texture.frag")
    discard_a = float(_one(r"if\s*\(\s*color\.a\s*<\s*(" + NUM + r")\s*\)", comp, "render_liquid_texture.frag"))
    a0, a1 = _one(r"alpha\s*=\s*smoothstep\(\s*(" + NUM + r")\s*,\s*(" + NUM + r")\s*,\s*color\.a\s*\)", comp,
                  "render_liquid_texture.frag")
    w0, w1 = _one(r"white\s*=\s*smoothstep\(\s*(" + NUM + r")\s*,\s*(" + NUM + r")\s*,\s*-color\.a\s*\)", comp,
                  "render_liquid_texture.frag")
    scale = float(_one(r"vec4\(\s*white\s*,\s*white\s*,\s*1\.0\s*,\s*(" + NUM + r")\s*\*\s*alpha\s*\)", comp,
                       "render_liquid_texture.frag"))
    rend = _read(root, "src/renderer.c")
    diam = set(re.findall(r"liquid_particle_diameter_pixels\s*=\s*gl_state\.screen_width\s*\*\s*(" + NUM + r")\s*;",
                          rend))
    if len(diam) != 1:
        raise ValueError(f"renderer.c: liquid sprite diameters {sorted(diam)}")
    liq = _read(root, "src/liquid_gl.c")
    red = re.search(r"#ifdef\s+RASPI\s+state->reduction\s*=\s*(\d+)\s*;\s*#else\s+state->reduction\s*=\s*(\d+)\s*;",
                    liq)
    if not red:
        raise ValueError("liquid_gl.c: texture reduction not found")
    return {"blur_weights_in_tap_order": weights, "blur_tap_order": order,
            "vertical_offsets": v_along, "vertical_cross_offsets": v_across,
            "horizontal_offsets": h_along, "horizontal_cross_offsets": h_across,
            "sprite_discard_r2": discard_r2, "sprite_intensity": [float(i0), float(i1)],
            "composite_discard_alpha": discard_a, "composite_alpha_edges": [float(a0), float(a1)],
            "composite_white_edges": [float(w0), float(w1)], "composite_alpha_scale": scale,
            "sprite_diameter_per_screen_width": float(diam.pop()),
            "texture_reduction": int(red.group(2))}


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else default_reference_root()
    c = read_constants(root)
    with open(OUT, "w") as f:
        json.dump(c, f, indent=1)
        f.write("\n")
    print(f"wrote {OUT}")


if __name__ == "__main__":
    main()
