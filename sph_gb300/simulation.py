"""Python host wrapper of the libsph_cuda fast API (include/sph_cuda.h).

`Simulation` owns one library handle: one single-device SPH domain whose
particle state stays in GPU memory between steps.  Every method maps to one
C-ABI call; arrays cross the boundary as host numpy buffers.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import (AABB, Counters, NeighborGrid, Param, PARTICLE_DTYPE, check, lib,
                   tunables)


def _f(a):
    return a.ctypes.data_as(_lib.c_float_p)


class Simulation:
    """One compute rank's domain on the GPU.

    params : dict of tunable_parameters fields (smoothing_radius = h)
    config : dict(box=(min_x, max_x, min_y, max_y), spacing, size_x, size_y,
             max_bucket, max_neighbors) -- the reference's grid set-up
             (fluid.c:173-176, 214-215)
    capacity : maximum particle count of the handle
    """

    def __init__(self, params: dict, config: dict, capacity: int):
        self._h = ctypes.c_void_p()
        p = Param()
        p.tunable_params = tunables(params)
        p.number_fluid_particles_global = capacity
        p.number_fluid_particles_local = capacity
        p.max_fluid_particle_index = capacity - 1
        p.number_halo_particles = 0
        b = AABB()
        b.min_x, b.max_x, b.min_y, b.max_y = (float(v) for v in config["box"])
        g = NeighborGrid()
        g.spacing = config["spacing"]
        g.size_x, g.size_y = config["size_x"], config["size_y"]
        g.max_bucket_size = config["max_bucket"]
        g.max_neighbors = config["max_neighbors"]
        check(lib().sph_cuda_create(ctypes.byref(self._h), ctypes.byref(p), ctypes.byref(b),
                                    ctypes.byref(g), int(capacity)))
        self.params = dict(params)
        self.config = dict(config)
        self.capacity = int(capacity)
        self.n = 0

    @classmethod
    def from_scene(cls, scene, capacity: int | None = None) -> "Simulation":
        sim = cls(scene.params.as_dict(), scene.config(), capacity or scene.n)
        sim.upload(scene.x, scene.y, scene.vx, scene.vy)
        return sim

    # -- lifecycle ---------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            lib().sph_cuda_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._h

    # -- state -------------------------------------------------------------
    def upload(self, x, y, vx=None, vy=None):
        arrs = [None if a is None else np.ascontiguousarray(a, np.float32) for a in (x, y, vx, vy)]
        n = len(arrs[0])
        check(lib().sph_cuda_upload_soa(self._h, *[None if a is None else _f(a) for a in arrs], n))
        self.n = n

    def init_lattice(self, blocks: list):
        """Generates the particles on the GPU (sph_cuda_init_lattice) from
        lattice-block dicts (n, cols, x0, y0, spacing, jitter, seed,
        counter0), e.g. the `lattice` entry of a synthetic scene's meta."""
        arr = (_lib.LatticeBlock * len(blocks))()
        for a, b in zip(arr, blocks):
            for k, _ in _lib.LatticeBlock._fields_:
                setattr(a, k, b[k])
        check(lib().sph_cuda_init_lattice(self._h, arr, len(blocks)))
        self.n = sum(int(b["n"]) for b in blocks)

    def upload_particles(self, particles: np.ndarray):
        """particles: structured array of PARTICLE_DTYPE (fluid_particle)."""
        a = np.ascontiguousarray(particles, PARTICLE_DTYPE)
        check(lib().sph_cuda_upload_particles(self._h, a.ctypes.data, len(a)))
        self.n = len(a)

    def download(self) -> dict:
        n = self.n
        out = {k: np.empty(n, np.float32) for k in ("x", "y", "v_x", "v_y", "density", "density_near")}
        check(lib().sph_cuda_download_soa(self._h, _f(out["x"]), _f(out["y"]), _f(out["v_x"]),
                                          _f(out["v_y"]), _f(out["density"]),
                                          _f(out["density_near"]), n))
        return out

    def download_particles(self) -> np.ndarray:
        a = np.zeros(self.n, PARTICLE_DTYPE)
        a["id"] = np.arange(self.n)
        check(lib().sph_cuda_download_particles(self._h, a.ctypes.data, self.n))
        return a

    def pack_coords(self, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty((self.n, 2), np.int16)
        check(lib().sph_cuda_pack_coords_short(self._h, out.ctypes.data_as(_lib.c_short_p), self.n))
        return out

    # -- stepping ------------------------------------------------------------
    def pack_coords_async(self, out: np.ndarray):
        """Starts the packed-coordinate copy into `out` ([n, 2] int16,
        page-locked); wait_coords(out) completes it."""
        check(lib().sph_cuda_pack_coords_async(self._h, out.ctypes.data_as(_lib.c_short_p), self.n))

    def wait_coords(self, out: np.ndarray):
        check(lib().sph_cuda_coords_wait(self._h, out.ctypes.data_as(_lib.c_short_p)))

    def step(self, params: dict | None = None, nsteps: int = 1):
        t = tunables(params or self.params)
        check(lib().sph_cuda_step(self._h, ctypes.byref(t), int(nsteps)))

    def set_scene_params(self, scene: int, params: dict):
        check(lib().sph_cuda_set_scene_params(self._h, int(scene), ctypes.byref(tunables(params))))

    def autotune(self, trial_steps: int = 3) -> list:
        """Picks the fastest launch shape per gather kernel, then long-row
        hit masks on or off (long_row_masks()), by timing graph-launched
        steps (advances the simulation by 50 * trial_steps steps); returns
        the 6 shape ints."""
        out = (ctypes.c_int * 6)()
        check(lib().sph_cuda_autotune(self._h, int(trial_steps), out))
        return list(out)

    def launch_shapes(self) -> list:
        out = (ctypes.c_int * 6)()
        check(lib().sph_cuda_get_launch_shapes(self._h, out))
        return list(out)

    def set_launch_shapes(self, shapes):
        arr = (ctypes.c_int * 6)(*[int(v) for v in shapes])
        check(lib().sph_cuda_set_launch_shapes(self._h, arr))

    def long_row_masks(self) -> bool:
        """Whether the density pass records hit masks for stencil rows of
        65..128 candidates (sph_cuda_set_long_row_masks)."""
        return bool(lib().sph_cuda_get_long_row_masks(self._h))

    def set_long_row_masks(self, on: bool):
        check(lib().sph_cuda_set_long_row_masks(self._h, 1 if on else 0))

    def step_split(self, before: dict | None, after: dict):
        """One step whose tunables switch after the prediction, where the
        reference's compute rank receives new ones (sph_cuda_step_split);
        `after` stays in force (and becomes this object's params)."""
        b = None if before is None else ctypes.byref(tunables(before))
        check(lib().sph_cuda_step_split(self._h, b, ctypes.byref(tunables(after))))
        self.params = dict(after)

    def step_schedule(self, params_list: list):
        arr = (_lib.TunableParameters * len(params_list))(*[tunables(p) for p in params_list])
        check(lib().sph_cuda_step_schedule(self._h, arr, len(params_list)))

    def save_state(self, path: str):
        """Checkpoint (sph_cuda_save_state)."""
        check(lib().sph_cuda_save_state(self._h, str(path).encode()))

    def load_state(self, path: str):
        """Resume from a checkpoint (sph_cuda_load_state)."""
        check(lib().sph_cuda_load_state(self._h, str(path).encode()))
        import struct
        with open(path, "rb") as f:
            self.n = struct.unpack("<i", f.read(16)[12:16])[0]

    def rebuild_neighbors(self):
        check(lib().sph_cuda_rebuild_neighbors(self._h))

    def synchronize(self):
        check(lib().sph_cuda_synchronize(self._h))

    # -- inspection ------------------------------------------------------------
    def scene_diagnostics(self) -> np.ndarray:
        """[nscenes, 3]: mean density, mean near density, kinetic energy per particle."""
        ns = int(lib().sph_cuda_num_scenes(self._h))
        out = np.zeros((ns, 3), np.float64)
        check(lib().sph_cuda_scene_diagnostics(self._h, out.ctypes.data_as(_lib.c_double_p)))
        return out

    def diagnostics(self) -> np.ndarray:
        out = np.zeros(3, np.float64)
        check(lib().sph_cuda_diagnostics(self._h, out.ctypes.data_as(_lib.c_double_p)))
        return out

    def counters(self) -> dict:
        c = Counters()
        check(lib().sph_cuda_get_counters(self._h, ctypes.byref(c)))
        return {k: getattr(c, k) for k, _ in Counters._fields_}

    def neighbor_lists(self):
        counts = np.zeros(max(self.n, 1), np.int32)
        total = ctypes.c_longlong(0)
        st = lib().sph_cuda_neighbor_lists(self._h, counts.ctypes.data_as(_lib.c_int_p), None, 0,
                                           ctypes.byref(total))
        if st not in (0, 4):
            check(st)
        ids = np.zeros(max(total.value, 1), np.int32)
        check(lib().sph_cuda_neighbor_lists(self._h, counts.ctypes.data_as(_lib.c_int_p),
                                            ids.ctypes.data_as(_lib.c_int_p), total.value,
                                            ctypes.byref(total)))
        return counts[:self.n].copy(), ids[:total.value].copy()

    def _probe(self, fn, params):
        """params None: the handle's own tunables (each scene's, for an
        ensemble)."""
        t = None if params is None else ctypes.byref(tunables(params))
        a = np.zeros(self.n, np.float32)
        b = np.zeros(self.n, np.float32)
        check(fn(self._h, t, _f(a), _f(b)))
        return a, b

    def probe_density(self, params: dict | None = None):
        return self._probe(lib().sph_cuda_probe_density, params)

    def probe_relaxation(self, params: dict | None = None):
        return self._probe(lib().sph_cuda_probe_relaxation, params)

    def probe_viscosity(self, params: dict | None = None):
        return self._probe(lib().sph_cuda_probe_viscosity, params)

    def kernel_times(self, params: dict | None = None) -> dict:
        """Runs ONE step with per-kernel CUDA events; {kernel name: ms}.
        params None keeps the tunables of the previous step."""
        t = None if params is None else ctypes.byref(tunables(params))
        ms = np.zeros(32, np.float32)
        cnt = ctypes.c_int(0)
        check(lib().sph_cuda_kernel_times(self._h, t, _f(ms), 32, ctypes.byref(cnt)))
        return {lib().sph_cuda_step_kernel_name(self._h, k).decode(): float(ms[k])
                for k in range(cnt.value)}

    def launches_per_step(self) -> int:
        return int(lib().sph_cuda_launches_per_step(self._h))

    def timer_start(self):
        check(lib().sph_cuda_timer_start(self._h))

    def timer_stop(self) -> float:
        """Milliseconds on the handle's stream since timer_start (synchronises)."""
        ms = ctypes.c_float(0.0)
        check(lib().sph_cuda_timer_stop(self._h, ctypes.byref(ms)))
        return float(ms.value)


    def render_liquid(self, width: int = 1920, height: int = 1080, alpha: bool = False):
        """The render rank's liquid image of the current particles:
        (height, width, 3) uint8, top row first; with alpha=True also the
        blurred half-resolution alpha texture (bottom row first)."""
        rgb = np.zeros((height, width, 3), np.uint8)
        a = np.zeros((height // 2, width // 2), np.uint8) if alpha else None
        check(lib().sph_cuda_render_liquid(self._h, int(width), int(height), rgb.ctypes.data,
                                           a.ctypes.data if alpha else None))
        return (rgb, a) if alpha else rgb

    # -- learned relaxation -------------------------------------------------
    def set_learned(self, model: "LearnedModel | None", threshold: float = 0.01):
        """Attaches a trained model (None detaches): particles whose
        predicted density error is at most `threshold` x rest density take
        the network's displacement, the rest the plain relaxation."""
        check(lib().sph_cuda_set_learned(self._h, None if model is None else model._l,
                                         float(threshold)))
        self._learned = model

    def learned_counts(self) -> tuple:
        """(particle-steps that used the network, particle-steps that fell
        back) since the model was attached."""
        a, b = ctypes.c_ulonglong(0), ctypes.c_ulonglong(0)
        check(lib().sph_cuda_learned_counts(self._h, ctypes.byref(a), ctypes.byref(b)))
        return int(a.value), int(b.value)

    def learned_features(self):
        """(features [n, 32] float32 by id, neighbour counts [n] int32, -1
        for particles that always take the plain relaxation) of the state
        the next step relaxes."""
        f = np.zeros((self.n, LearnedModel.IN), np.float32)
        c = np.zeros(self.n, np.int32)
        check(lib().sph_learned_features(self._h, _f(f), c.ctypes.data_as(_lib.c_int_p)))
        return f, c


class LearnedModel:
    """The learned relaxation's network (include/sph_learned.h): a 2-layer,
    width-128 GELU MLP over per-particle neighbour messages, BF16 on the
    tcgen05 tensor cores with FP32 accumulation and FP32 Adam."""

    IN, HIDDEN, OUT, MAX_NEIGHBORS = 32, 128, 16, 48

    def __init__(self, max_samples: int, seed: int = 0):
        self._l = ctypes.c_void_p()
        check(lib().sph_learned_create(ctypes.byref(self._l), int(max_samples), int(seed)))

    def close(self):
        if self._l is not None and self._l.value:
            check(lib().sph_learned_destroy(self._l))
        self._l = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @staticmethod
    def num_params() -> int:
        return int(lib().sph_learned_num_params())

    def collect(self, sim: Simulation, fraction: float = 1.0) -> int:
        n = ctypes.c_int(0)
        check(lib().sph_learned_collect(self._l, sim.handle, float(fraction), ctypes.byref(n)))
        return int(n.value)

    @property
    def num_samples(self) -> int:
        return int(lib().sph_learned_num_samples(self._l))

    def clear_samples(self):
        check(lib().sph_learned_clear_samples(self._l))

    def train(self, epochs: int, batch: int = 4096, lr: float = 1e-3) -> float:
        loss = ctypes.c_float(0.0)
        check(lib().sph_learned_train(self._l, int(epochs), int(batch), float(lr), ctypes.byref(loss)))
        return float(loss.value)

    def calibrate(self, sim: Simulation, epochs: int = 4, lr: float = 1e-3) -> float:
        loss = ctypes.c_float(0.0)
        check(lib().sph_learned_calibrate(self._l, sim.handle, int(epochs), float(lr),
                                          ctypes.byref(loss)))
        return float(loss.value)

    def get_params(self) -> np.ndarray:
        w = np.zeros(self.num_params(), np.float32)
        check(lib().sph_learned_get_params(self._l, _f(w)))
        return w

    def set_params(self, w: np.ndarray):
        w = np.ascontiguousarray(w, np.float32)
        if w.shape != (self.num_params(),):
            raise ValueError(f"expected {self.num_params()} parameters, got {w.shape}")
        check(lib().sph_learned_set_params(self._l, _f(w)))

    def forward(self, features: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(features, np.float32)
        n = x.shape[0]
        out = np.zeros((n, self.OUT), np.float32)
        check(lib().sph_learned_forward(self._l, _f(x), n, _f(out)))
        return out

    @staticmethod
    def unpack(w: np.ndarray) -> dict:
        """Named views of a flat parameter vector."""
        I, H, O = LearnedModel.IN, LearnedModel.HIDDEN, LearnedModel.OUT
        sizes = [("W1", (H, I)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("W3", (O, H)),
                 ("b3", (O,))]
        out, o = {}, 0
        for name, shp in sizes:
            k = int(np.prod(shp))
            out[name] = w[o:o + k].reshape(shp)
            o += k
        return out


def render_liquid(coords: np.ndarray, width: int = 1920, height: int = 1080):
    """The liquid image (and the half-resolution alpha texture) from packed
    short coordinates [n, 2] (sph_render_liquid)."""
    c = np.ascontiguousarray(coords, np.int16)
    rgb = np.zeros((height, width, 3), np.uint8)
    a = np.zeros((height // 2, width // 2), np.uint8)
    check(lib().sph_render_liquid(c.ctypes.data_as(_lib.c_short_p), int(c.shape[0]), int(width),
                                  int(height), rgb.ctypes.data, a.ctypes.data))
    return rgb, a


def write_ppm(path: str, rgb: np.ndarray):
    """Binary PPM (P6) of an RGB8 image, top row first."""
    h, w, _ = rgb.shape
    with open(path, "wb") as f:
        f.write(b"P6\n%d %d\n255\n" % (w, h))
        f.write(np.ascontiguousarray(rgb, np.uint8).tobytes())


def gemm_check(A: np.ndarray, B: np.ndarray) -> np.ndarray:
    """A [M, K] . B [N, K]^T on the tcgen05 tensor cores (BF16 in, FP32 out)."""
    A = np.ascontiguousarray(A, np.float32)
    B = np.ascontiguousarray(B, np.float32)
    M, K = A.shape
    N = B.shape[0]
    C = np.zeros((M, N), np.float32)
    check(lib().sph_learned_gemm_check(_f(A), _f(B), _f(C), M, N, K))
    return C


class Ensemble(Simulation):
    """Many independent scenes advanced together by one handle
    (sph_cuda_create_ensemble): one set of kernel launches per step covers
    every scene; particles are concatenated in scene order."""

    def __init__(self, scenes: list, max_bucket: int = 100, max_neighbors: int = 400):
        descs = (_lib.SceneDesc * len(scenes))()
        for d, sc in zip(descs, scenes):
            d.params = tunables(sc.params.as_dict())
            d.boundary.min_x, d.boundary.max_x, d.boundary.min_y, d.boundary.max_y = sc.box
            d.spacing = sc.spacing
            d.size_x, d.size_y = sc.size_x, sc.size_y
            d.n = sc.n
        self._h = ctypes.c_void_p()
        check(lib().sph_cuda_create_ensemble(ctypes.byref(self._h), descs, len(scenes),
                                             int(max_bucket), int(max_neighbors)))
        self.scenes = scenes
        self.offsets = np.concatenate([[0], np.cumsum([sc.n for sc in scenes])]).astype(np.int64)
        self.capacity = int(self.offsets[-1])
        self.params = None
        self.config = None
        self.n = 0

    def upload_scenes(self):
        cat = lambda k: np.concatenate([getattr(sc, k) for sc in self.scenes])  # noqa: E731
        self.upload(cat("x"), cat("y"), cat("vx"), cat("vy"))

    def step(self, params=None, nsteps: int = 1):
        if params is not None:
            raise ValueError("an ensemble takes per-scene tunables: use set_scene_params")
        check(lib().sph_cuda_step(self._h, None, int(nsteps)))

    def scene_slice(self, s: int) -> slice:
        return slice(int(self.offsets[s]), int(self.offsets[s + 1]))


class PinnedArray:
    """numpy view of page-locked host memory from sph_cuda_host_alloc."""

    def __init__(self, shape, dtype):
        self.dtype = np.dtype(dtype)
        nbytes = int(np.prod(shape)) * self.dtype.itemsize
        self._p = ctypes.c_void_p()
        check(lib().sph_cuda_host_alloc(ctypes.byref(self._p), nbytes))
        buf = (ctypes.c_byte * max(nbytes, 1)).from_address(self._p.value)
        self.array = np.frombuffer(buf, self.dtype, count=int(np.prod(shape))).reshape(shape)

    def free(self):
        if self._p.value:
            self.array = None
            lib().sph_cuda_host_free(self._p)
            self._p = ctypes.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass
