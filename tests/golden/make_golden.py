"""Generates the golden vectors in tests/golden/ from the REFERENCE's own
compiled step code (oracle/_ref/libsph_ref.so, built by `make -C oracle ref`
from the unmodified src/hash.c and src/fluid.c).

The reference has no tests or known-answer vectors of its own, so these
fixtures are its outputs on seeded synthetic inputs:

  cfg1.npz      3,000-particle dam break (96h x 48h): initial positions (pins
                the scene generator), states after 1, 10, 100 and 1,000 steps,
                per-step diagnostics of the 1,000-step run, hash_fluid lists
                and densities on the step-100 and step-1,000 positions.
  mover.npz     4,096-particle scaled dam break with the moving sphere mover
                (and a rectangle-mover variant): states, lists, densities.
  edges.npz     hand-placed cases: a bucket over its 100-particle cap, a
                particle exactly on x == max_x (cell aliasing), coincident
                particles, a pair at exactly r == h, one just beyond h.
  listcap.npz   five crowded cells whose half lists exceed the 400 cap.
  predict.npz   predict_positions with sphere and rectangle movers
                (boundaryConditions, fluid.c:656-744).

Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from sph_gb300 import scenes  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
STATE_FIELDS = ("x", "y", "v_x", "v_y", "density", "density_near")


def state(sim, prefix):
    s = sim.get()
    return {f"{prefix}_{k}": s[k] for k in STATE_FIELDS}


def lists_and_density(kind, x, y, params, config, prefix):
    z = np.zeros_like(x)
    sim = oracle.Sim(kind, x, y, z, z, params, config)
    counts, ids = sim.hash(compute_density=True)
    s = sim.get()
    return {f"{prefix}_counts": counts, f"{prefix}_ids": ids,
            f"{prefix}_rho": s["density"], f"{prefix}_rhon": s["density_near"]}


def make_cfg1():
    sc = scenes.config1()
    P, C = sc.params.as_dict(), sc.config()
    sim = oracle.Sim("ref", sc.x, sc.y, sc.vx, sc.vy, P, C)
    out = {"init_x": sc.x, "init_y": sc.y}
    diag = []
    done = 0
    for t in (1, 10, 100, 1000):
        diag.append(sim.step(t - done))
        done = t
        out.update(state(sim, f"s{t}"))
    out["diag"] = np.concatenate(diag)
    for t in (100, 1000):
        out.update(lists_and_density("ref", out[f"s{t}_x"], out[f"s{t}_y"], P, C, f"h{t}"))
    np.savez_compressed(os.path.join(OUT, "cfg1.npz"), **out)


def make_mover():
    out = {}
    for tag, mtype, w, hgt in (("sphere", scenes.SPHERE_MOVER, 16.0, 16.0),
                               ("rect", scenes.RECTANGLE_MOVER, 12.0, 6.0)):
        sc = scenes.config2(n=4096)
        sc.params.mover_type = mtype
        sc.params.mover_width, sc.params.mover_height = w, hgt
        P, C = sc.params.as_dict(), sc.config()
        sim = oracle.Sim("ref", sc.x, sc.y, sc.vx, sc.vy, P, C)
        mv = sc.mover_schedule(0, 100)
        out[f"{tag}_diag"] = sim.step(100, mover_xy=mv)
        out.update(state(sim, f"{tag}_s100"))
        out[f"{tag}_mover"] = mv
        out.update(lists_and_density("ref", out[f"{tag}_s100_x"], out[f"{tag}_s100_y"], P, C,
                                     f"{tag}_h100"))
    np.savez_compressed(os.path.join(OUT, "mover.npz"), **out)


EDGE_CONFIG = dict(box=(0.0, 16.0, 0.0, 16.0), spacing=1.0, size_x=16, size_y=16,
                   max_bucket=100, max_neighbors=400)


def edge_positions():
    rng = np.random.default_rng(7)
    pts = []
    # 130 particles in cell (3, 3): the bucket keeps the first 100 (hash.c:160)
    pts += list(zip(3.0 + rng.random(130) * 0.999, 3.0 + rng.random(130) * 0.999))
    # a loose lattice with a particle exactly on the right wall (aliases cell (0, gy+1))
    for j in range(6):
        for i in range(6):
            pts.append((10.2 + 0.55 * i, 8.1 + 0.6 * j))
    pts.append((16.0, 9.3))
    pts.append((15.6, 9.35))
    pts.append((0.3, 10.2))       # near the aliased cell (0, 10)
    # coincident particles and the exact-cutoff pair r == h (inclusive, hash.c:185)
    pts += [(6.25, 12.5), (6.25, 12.5), (6.75, 12.5)]
    pts += [(5.0, 5.5), (6.0, 5.5)]
    pts += [(5.0, 7.25), (5.0, 8.25000048)]      # just beyond h
    pts += [(1.0, 1.0), (1.0 + 0.5, 1.0 + 0.75)]
    a = np.array(pts, np.float32)
    return a[:, 0].copy(), a[:, 1].copy()


def listcap_positions():
    rng = np.random.default_rng(11)
    centres = [(8.9, 8.5), (8.9, 9.1), (9.1, 7.9), (9.1, 8.5), (9.1, 9.1)]
    xs, ys = [], []
    for cx, cy in centres:
        xs.append(cx + (rng.random(100) - 0.5) * 0.09)
        ys.append(cy + (rng.random(100) - 0.5) * 0.09)
    return np.concatenate(xs).astype(np.float32), np.concatenate(ys).astype(np.float32)


def make_edges():
    P = scenes.Params().as_dict()
    out = {}
    x, y = edge_positions()
    out.update(x=x, y=y)
    out.update(lists_and_density("ref", x, y, P, EDGE_CONFIG, "edge"))
    np.savez_compressed(os.path.join(OUT, "edges.npz"), **out)
    x, y = listcap_positions()
    out = dict(x=x, y=y)
    out.update(lists_and_density("ref", x, y, P, EDGE_CONFIG, "cap"))
    np.savez_compressed(os.path.join(OUT, "listcap.npz"), **out)


def make_predict():
    """predict_positions (fluid.c:507-523) on particles aimed into movers."""
    rng = np.random.default_rng(3)
    n = 2000
    x = (rng.random(n) * 15.8 + 0.1).astype(np.float32)
    y = (rng.random(n) * 15.8 + 0.1).astype(np.float32)
    vx = ((rng.random(n) - 0.5) * 10).astype(np.float32)
    vy = ((rng.random(n) - 0.5) * 10).astype(np.float32)
    out = dict(x=x, y=y, vx=vx, vy=vy)
    for tag, mtype, w, h in (("sphere", scenes.SPHERE_MOVER, 6.0, 6.0),
                             ("rect", scenes.RECTANGLE_MOVER, 7.0, 3.0)):
        p = scenes.Params(mover_type=mtype, mover_width=w, mover_height=h,
                          mover_center_x=8.0, mover_center_y=7.5, time_step=0.05)
        P = p.as_dict()
        sim = oracle.Sim("ref", x, y, vx, vy, P, EDGE_CONFIG)
        sim.call(2)
        s = sim.get()
        out[f"{tag}_x"], out[f"{tag}_y"] = s["x"], s["y"]
        out[f"{tag}_params"] = np.array([w, h, 8.0, 7.5, 0.05], np.float32)
    np.savez_compressed(os.path.join(OUT, "predict.npz"), **out)


def main():
    if not oracle.ref_available():
        oracle.build(ref=True)
    make_cfg1()
    make_mover()
    make_edges()
    make_predict()
    for f in sorted(os.listdir(OUT)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(OUT, f)))


if __name__ == "__main__":
    main()
