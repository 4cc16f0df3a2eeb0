"""Synthetic scenes for the SPH compute step (dam breaks and ensembles).

Every scene is reproducible from its seed with a documented generator
(splitmix64 counters -> uniform doubles), so the CUDA library and the CPU
oracle receive bit-identical float32 inputs.

Dam break (the reference's lattice fill, geometry.c:29-67, moved into a box
corner): particles on a square lattice of spacing 0.5h filling a block from
the box floor at the left wall, row-major from (0, 0), `cols` particles per
row, jittered by U(-0.01h, 0.01h) per axis, zero velocity.  Smoothing radius
h = 1, neighbour-grid spacing h (fluid.c:176), grid size ceil(box/h)
(fluid.c:214-215), bucket cap 100 and list cap 400 (fluid.c:174-175).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

SPHERE_MOVER = 0      # fluid.h:48
RECTANGLE_MOVER = 1   # fluid.h:49

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def splitmix64(seed: int, counters: np.ndarray) -> np.ndarray:
    """splitmix64 output for each counter value (uint64 array)."""
    with np.errstate(over="ignore"):
        z = np.uint64(seed) + (counters.astype(np.uint64) + np.uint64(1)) * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return z


def uniform(seed: int, counters: np.ndarray) -> np.ndarray:
    """Uniform doubles in [0, 1): top 53 bits of splitmix64."""
    return (splitmix64(seed, counters) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


@dataclass
class Params:
    """The reference's tunable_parameters (fluid.h:78-97), by field name."""
    rest_density: float = 1.3
    smoothing_radius: float = 1.0
    g: float = 9.8               # apply_gravity applies -g (fluid.c:403)
    k: float = 0.3
    k_near: float = 1.5
    k_spring: float = 10.0       # reference default, fluid.c:94
    sigma: float = 0.5
    beta: float = 0.1
    time_step: float = 1.0 / 60.0
    node_start_x: float = 0.0
    node_end_x: float = 0.0
    mover_center_x: float = -1000.0
    mover_center_y: float = -1000.0
    mover_width: float = 0.0
    mover_height: float = 0.0
    mover_type: int = SPHERE_MOVER
    kill_sim: int = 0
    active: int = 1

    FIELDS = ("rest_density", "smoothing_radius", "g", "k", "k_near", "k_spring", "sigma",
              "beta", "time_step", "node_start_x", "node_end_x", "mover_center_x",
              "mover_center_y", "mover_width", "mover_height")

    def as_dict(self) -> dict:
        d = {f: float(getattr(self, f)) for f in self.FIELDS}
        d.update(mover_type=int(self.mover_type), kill_sim=int(self.kill_sim), active=int(self.active))
        return d


@dataclass
class Scene:
    name: str
    x: np.ndarray          # float32 [n]
    y: np.ndarray
    vx: np.ndarray
    vy: np.ndarray
    box: tuple             # (min_x, max_x, min_y, max_y)
    params: Params
    spacing: float = 1.0
    size_x: int = 0
    size_y: int = 0
    max_bucket: int = 100
    max_neighbors: int = 400
    steps: int = 1000
    mover_period: float = 0.0     # steps; 0 = static mover
    mover_amplitude: float = 0.0
    mover_base: tuple = (0.0, 0.0)
    meta: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return int(self.x.shape[0])

    @property
    def cells(self) -> int:
        return self.size_x * self.size_y

    def mover_at(self, t: int) -> tuple:
        """Mover centre set before step t (float32 values)."""
        if self.mover_period <= 0.0:
            return (np.float32(self.params.mover_center_x), np.float32(self.params.mover_center_y))
        cx = self.mover_base[0] + self.mover_amplitude * math.sin(2.0 * math.pi * t / self.mover_period)
        return (np.float32(cx), np.float32(self.mover_base[1]))

    def mover_schedule(self, t0: int, nsteps: int) -> np.ndarray:
        """[nsteps, 2] float32 mover centres for steps t0 .. t0+nsteps-1."""
        out = np.empty((nsteps, 2), np.float32)
        for i in range(nsteps):
            out[i] = self.mover_at(t0 + i)
        return out

    def params_at(self, t: int) -> Params:
        p = Params(**{k: getattr(self.params, k) for k in Params.FIELDS},
                   mover_type=self.params.mover_type, kill_sim=0, active=1)
        p.mover_center_x, p.mover_center_y = (float(v) for v in self.mover_at(t))
        return p

    def config(self) -> dict:
        return dict(box=tuple(float(b) for b in self.box), spacing=float(self.spacing),
                    size_x=self.size_x, size_y=self.size_y, max_bucket=self.max_bucket,
                    max_neighbors=self.max_neighbors)


def dam_break(n: int, cols: int, box_w: float, box_h: float, seed: int, *, name: str,
              params: Params | None = None, lattice: float = 0.5, jitter: float = 0.01,
              x0: float = 0.0, y0: float = 0.0) -> Scene:
    """Lattice block of `n` particles, `cols` per row, from (x0, y0)."""
    i = np.arange(n, dtype=np.int64)
    row, col = np.divmod(i, cols)
    u = uniform(seed, np.arange(2 * n, dtype=np.uint64)).reshape(n, 2)
    jx = (u[:, 0] * 2.0 - 1.0) * jitter
    jy = (u[:, 1] * 2.0 - 1.0) * jitter
    x = (x0 + col * lattice + jx).astype(np.float32)
    y = (y0 + row * lattice + jy).astype(np.float32)
    p = params or Params()
    p.node_start_x = 0.0
    p.node_end_x = float(box_w)
    h = float(p.smoothing_radius)
    sc = Scene(name=name, x=x, y=y, vx=np.zeros(n, np.float32), vy=np.zeros(n, np.float32),
               box=(0.0, float(box_w), 0.0, float(box_h)), params=p, spacing=h,
               size_x=int(math.ceil(box_w / h)), size_y=int(math.ceil(box_h / h)))
    sc.meta = dict(lattice=dict(n=n, cols=cols, x0=float(x0), y0=float(y0), spacing=float(lattice),
                                jitter=float(jitter), seed=int(seed), counter0=0))
    return sc


def config1() -> Scene:
    """3,000-particle dam break in a 96h x 48h box (64 particles per row, 46
    full rows + 56), no mover, 1,000 steps, seed 1001."""
    s = dam_break(3000, 64, 96.0, 48.0, seed=1001, name="dam_break_3k_96x48")
    s.steps = 1000
    return s


def config2(n: int = 4_194_304) -> Scene:
    """4,194,304-particle dam break: box 3,590h x 1,795h keeps config 1's fill
    fraction (0.1627) and 2:1 aspect; 2,393 particles per row (x <= 1,196h),
    1,752 full rows + 1,768; sphere mover of width 16h (radius 8h, fluid.c:666)
    centred at (598 + 20 sin(2 pi t / 240), 438), 1,000 steps, seed 1002.

    Smaller `n` gives the same construction scaled by sqrt(n / 4,194,304)
    (box, columns, mover centre and amplitude; radius kept at 8h)."""
    if n == 4_194_304:
        box_w, box_h, cols = 3590.0, 1795.0, 2393
        base, amp = (598.0, 438.0), 20.0
    else:
        s = math.sqrt(n / 4_194_304)
        box_w, box_h = float(math.ceil(3590 * s)), float(math.ceil(1795 * s))
        cols = max(8, int(round(2393 * s)))
        base, amp = (round(598 * s, 3), round(438 * s, 3)), max(1.0, round(20 * s, 3))
    p = Params(mover_type=SPHERE_MOVER, mover_width=16.0, mover_height=16.0)
    sc = dam_break(n, cols, box_w, box_h, seed=1002, name=f"dam_break_{n}", params=p)
    sc.steps = 1000
    sc.mover_period = 240.0
    sc.mover_amplitude = amp
    sc.mover_base = base
    sc.params.mover_center_x, sc.params.mover_center_y = (float(v) for v in sc.mover_at(0))
    return sc


def ensemble_scene(seed: int, name: str, n_range=(1024, 65536)) -> Scene:
    """One scene of the batched ensemble: N = round(exp U(ln lo, ln hi))
    particles; box aspect a ~ U[1, 4] and fill fraction f ~ U[0.2, 0.5] give a
    box of area 0.25 N / f, W = sqrt(area a), H = W / a; the fluid is a
    lattice block (spacing 0.5h, jitter 0.01h) filling a rectangle of the
    box's aspect scaled by sqrt(f), at a uniform random position in the box;
    k ~ U[0.1, 0.5], k_near ~ U[1, 3], sigma ~ U[0, 1], the rest as the dam
    break; no mover.  Scene randoms use counters 0..7 of the seed, the jitter
    counters 8 onward."""
    u = uniform(seed, np.arange(8, dtype=np.uint64))
    lo, hi = math.log(n_range[0]), math.log(n_range[1])
    n = int(round(math.exp(lo + (hi - lo) * u[0])))
    a = 1.0 + 3.0 * u[1]
    f = 0.2 + 0.3 * u[2]
    area = 0.25 * n / f
    w = math.sqrt(area * a)
    h_box = w / a
    fw, fh = w * math.sqrt(f), h_box * math.sqrt(f)
    x0, y0 = u[6] * (w - fw), u[7] * (h_box - fh)
    cols = max(1, int(fw / 0.5))
    p = Params(k=0.1 + 0.4 * u[3], k_near=1.0 + 2.0 * u[4], sigma=float(u[5]))
    i = np.arange(n, dtype=np.int64)
    row, col = np.divmod(i, cols)
    ju = uniform(seed, np.arange(8, 8 + 2 * n, dtype=np.uint64)).reshape(n, 2)
    x = (x0 + col * 0.5 + (ju[:, 0] * 2.0 - 1.0) * 0.01).astype(np.float32)
    y = (y0 + row * 0.5 + (ju[:, 1] * 2.0 - 1.0) * 0.01).astype(np.float32)
    bw, bh = np.float32(w), np.float32(h_box)
    p.node_start_x, p.node_end_x = 0.0, float(bw)
    sc = Scene(name=name, x=x, y=y, vx=np.zeros(n, np.float32), vy=np.zeros(n, np.float32),
               box=(0.0, float(bw), 0.0, float(bh)), params=p, spacing=1.0,
               size_x=int(math.ceil(float(bw))), size_y=int(math.ceil(float(bh))))
    sc.meta = dict(aspect=a, fill=f,
                   lattice=dict(n=n, cols=cols, x0=float(x0), y0=float(y0), spacing=0.5, jitter=0.01,
                                seed=int(seed), counter0=8))
    return sc


def config3(nscenes: int = 512, n_range=(1024, 65536)) -> list:
    """The batched ensemble: 512 scenes (seeds 3000 + s), 500 steps."""
    out = []
    for s in range(nscenes):
        sc = ensemble_scene(3000 + s, f"ensemble_{s}", n_range)
        sc.steps = 500
        out.append(sc)
    return out


def learned_training_scenes(count: int = 200, n: int = 65_536, seed0: int = 4000) -> list:
    """Training trajectories of the learned relaxation: `count` dam breaks of
    config 2's construction at `n` particles (mover held at its t = 0
    position), each with k ~ U[0.1, 0.5], k_near ~ U[1, 3], sigma ~ U[0, 1]
    drawn from counters 0..2 of seed seed0 + s (the ensemble's ranges)."""
    out = []
    for s in range(count):
        sc = config2(n)
        u = uniform(seed0 + s, np.arange(3, dtype=np.uint64))
        sc.params.k = float(0.1 + 0.4 * u[0])
        sc.params.k_near = float(1.0 + 2.0 * u[1])
        sc.params.sigma = float(u[2])
        sc.mover_period = 0.0
        sc.name = f"learned_train_{s}"
        out.append(sc)
    return out


def _reflect(v: np.ndarray, lo: float, hi: float) -> np.ndarray:
    """Folds values back into [lo, hi] (two reflections, then a clip)."""
    for _ in range(2):
        v = np.where(v < lo, 2 * lo - v, v)
        v = np.where(v > hi, 2 * hi - v, v)
    return np.clip(v, lo, hi)


def skewed_scene(seed: int, name: str, n_range=(512, 32768)) -> Scene:
    """One scene of the skewed ensemble (config 5), before settling: N =
    round(exp U(ln lo, ln hi)) particles in a box of area N h^2 (fill 0.25 at
    the lattice spacing 0.5h) with aspect W/H ~ U[1, 2].  A fraction
    U[0.5, 0.8] of them forms the pile: a jittered 0.5h lattice across the
    whole box width from the floor.  The rest forms 1-6 Gaussian blobs
    (sigma ~ U[3, 10]h, at most W/4, widened where needed so that the blob's
    peak density stays at most 4 particles per h^2; with overlaps and
    counting noise the fullest cells hold about 12), centred above the pile;
    blob particles are kept in the box by reflection at the walls.  k ~
    U[0.1, 0.5], k_near ~ U[1, 3], sigma ~ U[0, 1].  Scene randoms use
    counters 0..15 of the seed (blob b: 8 + 2b, 9 + 2b; b < 4 share the rest
    as rescaled draws), the lattice jitter the next 2 N_pile counters, the
    blob offsets the 2 N_blob after them.  `x`, `y` hold the pile and
    meta['blob_x'], meta['blob_y'] the blob particles."""
    u = uniform(seed, np.arange(16, dtype=np.uint64))
    lo, hi = math.log(n_range[0]), math.log(n_range[1])
    n = int(round(math.exp(lo + (hi - lo) * u[0])))
    nblobs = 1 + min(5, int(u[1] * 6))
    pile_frac = 0.5 + 0.3 * u[2]
    aspect = 1.0 + u[3]
    p = Params(k=0.1 + 0.4 * u[4], k_near=1.0 + 2.0 * u[5], sigma=float(u[6]))
    w = math.sqrt(n * aspect)
    h_box = w / aspect
    n_pile = int(round(n * pile_frac))
    n_blob = n - n_pile
    cols = max(1, int(w / 0.5) - 1)
    i = np.arange(n_pile, dtype=np.int64)
    row, col = np.divmod(i, cols)
    ju = uniform(seed, np.arange(16, 16 + 2 * n_pile, dtype=np.uint64)).reshape(n_pile, 2)
    x = (0.25 + col * 0.5 + (ju[:, 0] * 2.0 - 1.0) * 0.01).astype(np.float32)
    y = (0.25 + row * 0.5 + (ju[:, 1] * 2.0 - 1.0) * 0.01).astype(np.float32)
    pile_top = 0.25 + (int(row.max()) + 1 if n_pile else 0) * 0.5
    # blobs
    g = uniform(seed, np.arange(16 + 2 * n_pile, 16 + 2 * n_pile + 2 * n_blob,
                                dtype=np.uint64)).reshape(max(n_blob, 0), 2)
    r = np.sqrt(-2.0 * np.log(np.maximum(g[:, 0], 1e-300)))
    gx, gy = r * np.cos(2 * math.pi * g[:, 1]), r * np.sin(2 * math.pi * g[:, 1])
    counts = [n_blob // nblobs + (1 if b < n_blob % nblobs else 0) for b in range(nblobs)]
    bx, by, o = [], [], 0
    blobs = []
    for b in range(nblobs):
        ua, ub = (u[8 + 2 * b], u[9 + 2 * b]) if b < 4 else ((u[7] * (b + 1)) % 1.0, (u[15] * (b + 2)) % 1.0)
        sig = min(3.0 + 7.0 * ua, w / 4.0)
        sig = max(sig, math.sqrt(counts[b] / (2 * math.pi * 4.0)))
        cx = sig + (w - 2 * sig) * ub if w > 2 * sig else w / 2
        room = max(0.0, h_box - pile_top - 3 * sig)
        cy = min(h_box - sig, pile_top + 1.5 * sig + room * ((ua + ub) % 1.0))
        k = counts[b]
        bx.append(_reflect(cx + sig * gx[o:o + k], 0.05, w - 0.05))
        by.append(_reflect(cy + sig * gy[o:o + k], 0.05, h_box - 0.05))
        blobs.append(dict(n=k, sigma=sig, centre=(cx, cy)))
        o += k
    p.node_start_x, p.node_end_x = 0.0, float(np.float32(w))
    sc = Scene(name=name, x=x, y=y, vx=np.zeros(n_pile, np.float32), vy=np.zeros(n_pile, np.float32),
               box=(0.0, float(np.float32(w)), 0.0, float(np.float32(h_box))), params=p, spacing=1.0,
               size_x=int(math.ceil(float(np.float32(w)))), size_y=int(math.ceil(float(np.float32(h_box)))))
    sc.meta = dict(n_total=n, n_pile=n_pile, pile_top=pile_top, blobs=blobs,
                   lattice=dict(n=n_pile, cols=cols, x0=0.25, y0=0.25, spacing=0.5, jitter=0.01,
                                seed=int(seed), counter0=16),
                   blob_x=np.concatenate(bx).astype(np.float32) if bx else np.zeros(0, np.float32),
                   blob_y=np.concatenate(by).astype(np.float32) if by else np.zeros(0, np.float32))
    sc.steps = 500
    return sc


def config5(nscenes: int = 2048, n_range=(512, 32768)) -> list:
    """The skewed ensemble before settling: 2,048 scenes (seeds 5000 + s)."""
    return [skewed_scene(5000 + s, f"skewed_{s}", n_range) for s in range(nscenes)]


SETTLE_STEPS = 300


def settle_and_drop(piles: list, steps: int = SETTLE_STEPS) -> list:
    """Settles every scene's pile with the plain method on the GPU (one
    batched ensemble, `steps` steps, tunables of each scene), then adds the
    blob particles at rest: the scenes of config 5."""
    from .simulation import Ensemble
    e = Ensemble(piles)
    e.upload_scenes()
    e.step(None, steps)
    st = e.download()
    e.close()
    out = []
    for k, sc in enumerate(piles):
        sl = e.scene_slice(k)
        bx, by = sc.meta["blob_x"], sc.meta["blob_y"]
        nb = bx.shape[0]
        full = Scene(name=sc.name, x=np.concatenate([st["x"][sl], bx]).astype(np.float32),
                     y=np.concatenate([st["y"][sl], by]).astype(np.float32),
                     vx=np.concatenate([st["v_x"][sl], np.zeros(nb, np.float32)]).astype(np.float32),
                     vy=np.concatenate([st["v_y"][sl], np.zeros(nb, np.float32)]).astype(np.float32),
                     box=sc.box, params=sc.params, spacing=sc.spacing, size_x=sc.size_x,
                     size_y=sc.size_y, steps=sc.steps)
        full.meta = {k: v for k, v in sc.meta.items() if k != "lattice"}
        full.meta["settle_steps"] = steps
        out.append(full)
    return out


def slab_columns(columns: int, nslabs: int) -> list:
    """The 1-D x-slab decomposition of a lattice block of `columns` particle
    columns over `nslabs` compute ranks, as partitionProblem
    (geometry.c:101-160) cuts it: floor(columns / nslabs) columns each, the
    remainder one more each to the leftmost slabs.  Returns [(first column,
    number of columns)] per slab."""
    equal = columns // nslabs
    remaining = columns - equal * nslabs
    out, first = [], 0
    for s in range(nslabs):
        length = equal + (1 if s < remaining else 0)
        out.append((first, length))
        first += length
    return out


def slab_indices(sc: Scene, slab: int, nslabs: int) -> np.ndarray:
    """Particle indices of x-slab `slab` of a lattice-block scene (by the
    particle's lattice column, as the reference assigns particles to ranks
    at construction)."""
    lat = sc.meta["lattice"]
    first, length = slab_columns(int(lat["cols"]), nslabs)[slab]
    col = np.arange(sc.n, dtype=np.int64) % int(lat["cols"])
    return np.nonzero((col >= first) & (col < first + length))[0]


def algorithmic_bytes_per_step(n: int, cells: int) -> int:
    """Canonical algorithmic HBM bytes of one step: 216 B per particle
    (viscosity+predict 40, cell build on predicted positions 68, density 16,
    relaxation+update 40, cell build on relaxed positions 52) + 16 B per
    cell (cell start/count written and read by both builds)."""
    return 216 * n + 16 * cells
