"""Benchmark: particle-steps/s of the SPH compute step on GB300.

Workload: the 4,194,304-particle dam break with the moving sphere mover
(box 3,590h x 1,795h, h = 1; sph_gb300.scenes.config2).  A "step" is one
full reference step (fluid.c:273-348) over all particles.  The timed steps
continue the simulation after the warm-up steps (steps W .. W+K-1 of the
dam break), each step with its own mover position.

  value   device-resident throughput: CUDA events on the library's stream
          around K graph-launched steps (per-step tunables copied from pinned
          memory, as the reference receives them).
  e2e     the same metric through the C ABI from host buffers: upload of the
          particle state from host memory, then per step the tunables
          host->device and the packed render coordinates (fluid.c:356-362)
          device->host into pinned memory; wall clock around all of it.
  roofline  the dominant kernel's algorithmic bytes / its CUDA-event time,
          against the measured HBM copy bandwidth.
  cpu_baseline  the oracle's restatement of the reference step (Gauss-Seidel,
          single thread) on a bounded sample of the same construction.
  learned the learned-relaxation step on the same scene: a network trained
          (in the same run, untimed) on 200 plain-method trajectories of
          65,536-particle dam breaks with randomised stiffness and viscosity,
          run with the plain relaxation as fallback where its predicted
          density error exceeds 1% of the rest density; its throughput, its
          RMS density error against the plain step, and the tensor-core
          roofline of its MLP kernel.

--impl reference runs the reference's CPU step instead (the compiled
reference where present, else the restatement) on all host cores.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# Algorithmic bytes per particle (and per cell) of each kernel: the reads and
# writes its pass needs, neighbour reads served on chip not counted.  The
# three gathers use the per-pass figures of the canonical step budget
# (216 B per particle + 16 B per cell); the hit masks the density pass hands
# to the relaxation (24 B written, 24 B read per particle) are an
# implementation choice and are not counted as algorithmic.
ALG_BYTES = {
    "viscosity_predict": (40, 0),   # R pos, vel 16; W pos, prev, key+rank 24
    "cell_starts_1": (0, 12),       # R count, W start, W zero
    "cell_scatter_1": (20, 0),      # R key+rank 8, id 4, start 4; W slot 4
    "cell_permute_1": (52, 0),      # R key+rank 8, slots 4, id 4, pos 8, prev 8; W id, pos, prev 20
    "density": (16, 0),             # R pos 8; W rho, rho_near 8
    "relax_update": (40, 0),        # R pos, rho, prev 24; W pos, vel 16
    "cell_starts_2": (0, 12),
    "cell_scatter_2": (20, 0),
    "cell_permute_2": (52, 0),      # R key+rank, slots, id, pos, vel; W id, pos, vel
}


# MMA work of one network row: 32 -> 128 -> 128 -> 16 (multiply-adds x 2).
MLP_FLOPS_PER_ROW = 2 * (32 * 128 + 128 * 128 + 128 * 16)


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def load_tensor_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["bf16_tflops"]), "measured (burst)"
    except Exception:
        return 1900.0, "fallback"


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int = 0):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            for line in open(self.path):
                f = [v.strip() for v in line.split(",")]
                if len(f) >= 9:
                    rows.append(f)
        except Exception:
            pass
        finally:
            if self.path and os.path.exists(self.path):
                os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}

        def num(v):
            try:
                return float(v)
            except ValueError:
                return None
        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        mx = [num(r[2]) for r in rows if num(r[2]) is not None]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for i, nm in enumerate(names):
                if r[5 + i].lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows),
                "power_w_max": max((num(r[3]) or 0.0) for r in rows)}


def dist_setup():
    """One process per GPU under torchrun: each rank sees only its GPU.
    Ranks are independent replicas (the path does not shard); gloo carries
    only the barrier and the max-over-ranks time."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        vis = os.environ.get("CUDA_VISIBLE_DEVICES")
        devs = vis.split(",") if vis else [str(i) for i in range(64)]
        os.environ["CUDA_VISIBLE_DEVICES"] = devs[local]
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(world, v: float) -> float:
    if world <= 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_kind():
    import oracle
    if not os.path.exists(oracle.PORT_LIB):
        oracle.build(ref=False)
    return ("ref", "reference") if oracle.ref_available() else ("port", "port")


def time_cpu_slab(n: int, slab: int, nslabs: int, warmup: int, steps: int, kind: str):
    """One compute rank of the reference's decomposition of the dam break:
    x-slab `slab` of `nslabs` (geometry.c:101-160), its particles stepped by
    the reference's single-rank step loop (fluid.c:273-348) in the global
    box and grid, with the global mover schedule.  `warmup` untimed steps
    (the first has no viscosity, fluid.c:202), then `steps` timed ones.
    Returns (particles, seconds)."""
    import oracle
    from sph_gb300 import scenes
    sc = scenes.config2(n=n)
    idx = scenes.slab_indices(sc, slab, nslabs)
    sim = oracle.Sim(kind, sc.x[idx], sc.y[idx], sc.vx[idx], sc.vy[idx], sc.params.as_dict(),
                     sc.config())
    mv = sc.mover_schedule(0, warmup + steps)
    sim.step(warmup, mv[:warmup])
    t0 = time.perf_counter()
    sim.step(steps, mv[warmup:])
    dt = time.perf_counter() - t0
    sim.close()
    return len(idx), dt


def _slab_worker(args):
    return time_cpu_slab(*args)


def cpu_baseline_single(n, cores_hint, steps=12):
    """The reference step on one host core: the middle x-slab (the one the
    mover stirs) of the dam break cut into as many slabs as the host has
    cores, 12 steps after one untimed step."""
    kind, label = cpu_kind()
    nslabs = max(1, cores_hint)
    slab = nslabs // 2
    m, dt = time_cpu_slab(n, slab, nslabs, 1, steps, kind)
    return {"value": m * steps / dt, "unit": "particle-steps/s", "cores": 1, "kind": label,
            "sample": f"x-slab {slab} of the {n}-particle dam break cut into {nslabs} slabs as "
                      f"partitionProblem cuts it (geometry.c:101-160): {m} particles, {steps} steps "
                      f"after one untimed step, reference step order (Gauss-Seidel), single thread, "
                      f"-O2 -ffp-contract=off; no halo exchange"}


def run_reference(args, world, rank):
    """The reference's CPU step on all host cores, on the same dam break:
    the scene is cut into one x-slab per core exactly as partitionProblem
    (geometry.c:101-160) assigns particle columns to compute ranks, and each
    core runs its slab's single-rank step loop (fluid.c:273-348) for W
    untimed and K timed steps.  MPI is absent on the host, so the slabs do
    not exchange halos or migrants (communication.c): each slab is stepped as
    its own domain in the global box, an upper bound of the reference's
    multi-rank throughput.  value = all slabs' particles x K / the slowest
    slab's time."""
    if rank != 0:
        return
    import multiprocessing as mp
    kind, label = cpu_kind()
    cores = os.cpu_count() or 1
    K, W = args.steps, args.warmup
    ctx = mp.get_context("spawn")
    work = [(args.n, s, cores, W, K, kind) for s in range(cores)]
    t0 = time.perf_counter()
    with ctx.Pool(cores) as pool:
        res = pool.map(_slab_worker, work)
    wall = time.perf_counter() - t0
    total = sum(m for m, _ in res)
    busy = max(dt for _, dt in res)
    value = total * K / busy
    sizes = [m for m, _ in res]
    line = {"metric": "particle-steps/s", "value": value, "unit": "particle-steps/s",
            "impl": "reference", "n_gpus": args.gpus, "steps": K, "warmup": W,
            "ms_per_step": 1e3 * busy / K, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"dam break, {total} particles, box 3,590h x 1,795h, moving sphere "
                                   f"mover r=8h, plain method (reference step order)",
                       "particles": total, "slabs": cores, "slab_particles": [min(sizes), max(sizes)],
                       "steps_timed": f"{W}..{W + K - 1}", "wall_s": wall},
            "cpu_baseline": {"value": value, "unit": "particle-steps/s", "cores": cores, "kind": label,
                             "sample": f"the whole workload: {cores} x-slabs cut as partitionProblem cuts "
                                       f"them (geometry.c:101-160), one per core, each the reference's "
                                       f"single-rank step loop (fluid.c:273-348), steps {W}..{W + K - 1}; "
                                       f"no halo exchange or migration between slabs (no MPI on the host)"},
            "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def traffic_per_launch(kernel: str, n: int):
    """DRAM bytes per launch of `kernel` scaled from the committed ncu capture."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        d = json.load(open(p))
        k = d["kernels"][kernel]
        return k["dram_bytes"] * n / d["particles"]
    except Exception:
        return None


SMS, SCHEDULERS_PER_SM = 152, 4


def issue_bound(kernel: str, n: int, kernel_ms: float, sm_mhz):
    """The kernel's instruction-issue roofline: its warp instructions per
    launch (a committed single-launch ncu capture, scaled by particles) over
    its CUDA-event time, against one warp instruction per scheduler per
    clock on every SM at the SM clock sampled during the run."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        d = json.load(open(p))
        inst = d["kernels"][kernel]["warp_instructions"] * n / d["particles"]
    except Exception:
        return None
    mhz = sm_mhz or 2070.0
    achieved = inst / (kernel_ms / 1e3)
    peak = SMS * SCHEDULERS_PER_SM * mhz * 1e6
    return {"bound": "issue", "warp_instructions_per_launch": inst, "achieved": achieved,
            "peak": peak, "unit": "warp instructions/s", "frac": achieved / peak,
            "sm_mhz": mhz, "source": "profiles/traffic.json (ncu smsp__inst_executed.sum)"}


class DamBreak:
    """The 4,194,304-particle dam break with the moving sphere mover."""

    def __init__(self, n):
        from sph_gb300 import scenes
        self.sc = scenes.config2(n=n)
        self.n, self.cells = self.sc.n, self.sc.cells
        self.name = (f"dam break, {self.n} particles, box {self.sc.box[1]:g}h x {self.sc.box[3]:g}h, "
                     f"moving sphere mover r=8h, plain method")
        self.params = {}

    def p(self, t):
        if t not in self.params:
            self.params[t] = self.sc.params_at(t).as_dict()
        return self.params[t]

    def fresh(self):
        from sph_gb300 import Simulation
        return Simulation.from_scene(self.sc)

    def blank(self):
        """A handle for the scene with no particles uploaded yet."""
        from sph_gb300 import Simulation
        return Simulation(self.sc.params.as_dict(), self.sc.config(), self.sc.n)

    def state(self):
        """The initial x, y, vx, vy (host arrays)."""
        return self.sc.x, self.sc.y, self.sc.vx, self.sc.vy

    def advance(self, sim, t0, k):
        sim.step_schedule([self.p(t) for t in range(t0, t0 + k)])

    tunables_bytes = 64  # one tunable_parameters record per step (fluid.h:78-97)

    def step_one(self, sim, t):
        sim.step(self.p(t))

    def tune(self, sim):
        return sim.autotune(3)  # 144 steps (3 interleaved rounds) with the last step's tunables

    def cpu_sample(self, args):
        return cpu_baseline_single(self.n, os.cpu_count() or 1, args.cpu_steps)


class EnsembleWork:
    """512 independent scenes of 1,024-65,536 particles in one step."""

    def __init__(self, nscenes):
        from sph_gb300 import scenes
        self.scs = scenes.config3(nscenes)
        self.n = sum(s.n for s in self.scs)
        self.cells = sum(s.cells for s in self.scs)
        self.name = (f"batched ensemble, {nscenes} scenes, {self.n} particles (1,024-65,536 per "
                     f"scene, log-uniform), plain method")

    def fresh(self):
        from sph_gb300 import Ensemble
        e = Ensemble(self.scs)
        e.upload_scenes()
        return e

    def blank(self):
        from sph_gb300 import Ensemble
        return Ensemble(self.scs)

    def state(self):
        import numpy as np
        return tuple(np.concatenate([getattr(sc, k) for sc in self.scs]) for k in ("x", "y", "vx", "vy"))

    def advance(self, sim, t0, k):
        sim.step(None, k)

    tunables_bytes = 0  # the scenes keep their tunables

    def step_one(self, sim, t):
        sim.step(None, 1)

    def tune(self, sim):
        return sim.autotune(3)  # 144 steps (3 interleaved rounds)

    def cpu_sample(self, args):
        import oracle
        kind, label = cpu_kind()
        sample = self.scs[:16]
        steps = max(2, args.cpu_steps // 2)
        total = 0.0
        for sc in sample:
            sim = oracle.Sim(kind, sc.x, sc.y, sc.vx, sc.vy, sc.params.as_dict(), sc.config())
            sim.step(1)
            t0 = time.perf_counter()
            sim.step(steps)
            total += time.perf_counter() - t0
            sim.close()
        np_ = sum(s.n for s in sample)
        return {"value": np_ * steps / total, "unit": "particle-steps/s", "cores": 1, "kind": label,
                "sample": f"the first 16 scenes of the ensemble ({np_} particles), {steps} steps each "
                          f"after one untimed step, reference step order, single thread"}


def train_learned(args):
    """Trains the learned relaxation on plain-method trajectories: one
    batched ensemble of `train_scenes` dam breaks of `train_n` particles
    (randomised k, k_near, sigma), sampled every 10 steps; then calibrates
    its density-error output on one more trajectory's state."""
    from sph_gb300 import Ensemble, LearnedModel, Simulation, scenes
    t0 = time.perf_counter()
    tr = scenes.learned_training_scenes(args.train_scenes, args.train_n)
    total = sum(s.n for s in tr)
    every, steps = 10, args.train_steps
    frac = min(1.0, args.train_samples / (total * (steps // every)))
    m = LearnedModel(int(args.train_samples * 1.1) + 2 * args.train_n, seed=20261)
    e = Ensemble(tr)
    e.upload_scenes()
    for t in range(0, steps, every):
        e.step(None, every)
        m.collect(e, frac)
    e.close()
    t_collect = time.perf_counter() - t0
    losses = []
    for ep in range(args.train_epochs):
        lr = 1e-3 if ep < args.train_epochs - 2 else 3e-4
        losses.append(m.train(1, 4096, lr))
    cal_sc = scenes.learned_training_scenes(1, args.train_n, seed0=4000 + args.train_scenes)[0]
    with Simulation.from_scene(cal_sc) as s:
        s.step(cal_sc.params.as_dict(), 200)
        cal_loss = m.calibrate(s, epochs=4)
    info = {"trajectories": len(tr), "particles_per_trajectory": args.train_n,
            "steps_per_trajectory": steps, "samples": m.num_samples, "sample_every": every,
            "epochs": args.train_epochs, "loss_per_epoch": [round(v, 6) for v in losses],
            "calibration_loss": cal_loss, "collect_s": t_collect,
            "train_s": time.perf_counter() - t0 - t_collect}
    m.clear_samples()
    return m, info


def run_learned(args, work, plain_ms, shapes, long_masks=False):
    """The learned step on the dam break: throughput (CUDA events around
    graph-launched steps), one-step RMS density error against the plain step
    from the same state, the fallback share, and a 1,000-step trajectory's
    mean density and kinetic energy against the plain method's."""
    import numpy as np
    model, info = train_learned(args)
    thr = args.learned_threshold
    K, W = args.steps, args.warmup
    sim = work.fresh()
    sim.set_launch_shapes(shapes)
    sim.set_long_row_masks(long_masks)
    work.advance(sim, 0, W)
    sim.set_learned(model, thr)
    work.advance(sim, W, 5)
    sim.synchronize()
    with ClockSampler(0) as clk:
        sim.timer_start()
        work.advance(sim, W + 5, K)
        ms = sim.timer_stop()
    clocks = clk.summary()
    used, fell = sim.learned_counts()
    kt_runs = [sim.kernel_times(None) for _ in range(5)]
    ktimes = {k: statistics.median(r[k] for r in kt_runs) for k in kt_runs[0]}
    sim.close()
    n = work.n
    peak, peak_kind = load_tensor_peak()
    flops = MLP_FLOPS_PER_ROW * n
    achieved = flops / (ktimes["mlp"] / 1e3) / 1e12

    # one-step density error against the plain step from the same state
    t_state = 200
    a, b = work.fresh(), work.fresh()
    work.advance(a, 0, t_state)
    work.advance(b, 0, t_state)
    b.set_learned(model, thr)
    work.step_one(a, t_state)
    work.step_one(b, t_state)
    pa = work.p(t_state + 1)
    ra, _ = a.probe_density(pa)
    rb, _ = b.probe_density(pa)
    rest = work.sc.params.rest_density
    rms = float(np.sqrt(np.mean((ra.astype(np.float64) - rb) ** 2)) / rest)
    u1, f1 = b.learned_counts()
    # trajectories: plain vs learned over the scene's 1,000 steps
    traj = None
    if not args.no_trajectory:
        steps = work.sc.steps - t_state - 1
        work.advance(a, t_state + 1, steps)
        work.advance(b, t_state + 1, steps)
        da, db = a.diagnostics(), b.diagnostics()
        traj = {"steps": work.sc.steps, "plain": {"mean_density": da[0], "kinetic_energy": da[2]},
                "learned": {"mean_density": db[0], "kinetic_energy": db[2]},
                "mean_density_rel_diff": abs(db[0] - da[0]) / da[0],
                "kinetic_energy_rel_diff": abs(db[2] - da[2]) / max(abs(da[2]), 1e-30)}
    a.close()
    b.close()
    model.close()
    return {"value": n * K / (ms / 1e3), "unit": "particle-steps/s", "ms_per_step": ms / K,
            "vs_plain": (plain_ms) / (ms / K), "threshold_rest_density": thr,
            "network_share": used / max(1, used + fell),
            "rms_density_error_one_step": rms, "one_step_network_share": u1 / max(1, u1 + f1),
            "trajectory": traj, "training": info, "clocks": clocks,
            "roofline": {"bound": "tensor", "kernel": "mlp", "achieved": achieved, "peak": peak,
                         "unit": "TFLOP/s", "frac": achieved / peak, "peak_source": peak_kind,
                         "flops_per_launch": flops},
            "kernel_ms": {k: round(v, 5) for k, v in ktimes.items()}}


def run_skewed(args, world, rank):
    """Learned relaxation + batching under skew: 2,048 scenes (settled piles
    with Gaussian blobs dropped on them) in one graph-captured step with the
    learned relaxation, against the same ensemble with the plain step."""
    import numpy as np

    from sph_gb300 import Ensemble, scenes
    piles = scenes.config5(args.scenes)
    t0 = time.perf_counter()
    scs = scenes.settle_and_drop(piles, scenes.SETTLE_STEPS)
    t_settle = time.perf_counter() - t0
    n = sum(s.n for s in scs)
    cells = sum(s.cells for s in scs)
    model, info = train_learned(args)
    K, W = args.steps, args.warmup

    def fresh(learned):
        e = Ensemble(scs)
        e.upload_scenes()
        if learned:
            e.set_learned(model, args.learned_threshold)
        return e

    res = {}
    for label in ("plain", "learned"):
        # shapes tuned on a copy at the middle of the timed window
        tuner = fresh(label == "learned")
        tuner.step(None, W + K // 2)
        shapes = tuner.autotune(3)
        long_masks = tuner.long_row_masks()
        tuner.close()
        e = fresh(label == "learned")
        e.set_launch_shapes(shapes)
        e.set_long_row_masks(long_masks)
        e.step(None, W)
        e.synchronize()
        barrier(world)
        with ClockSampler(0) as clk:
            e.timer_start()
            e.step(None, K)
            ms = e.timer_stop()
        ms = max_over_ranks(world, ms)
        kt = [e.kernel_times(None) for _ in range(3)]
        res[label] = {"ms": ms, "clocks": clk.summary(), "shapes": shapes, "long_masks": long_masks,
                      "launches": e.launches_per_step() * K,
                      "kernel_ms": {k: round(statistics.median(r[k] for r in kt), 5) for k in kt[0]},
                      "counts": e.learned_counts() if label == "learned" else None}
        e.close()
    # one-step density error against the plain step from the same state
    a, b = fresh(False), fresh(False)
    a.step(None, 100)
    b.step(None, 100)
    b.set_learned(model, args.learned_threshold)
    a.step(None, 1)
    b.step(None, 1)
    used, fell = b.learned_counts()
    # densities of the post-step positions (the ensemble's own tunables)
    da, _ = a.probe_density()
    db, _ = b.probe_density()
    rest = scs[0].params.rest_density
    rms = float(np.sqrt(np.mean((da.astype(np.float64) - db) ** 2)) / rest)
    a.close()
    b.close()
    model.close()
    L, P = res["learned"], res["plain"]
    value = world * n * K / (L["ms"] / 1e3)
    peak, peak_kind = load_tensor_peak()
    mlp_ms = L["kernel_ms"]["mlp"]
    achieved = MLP_FLOPS_PER_ROW * n / (mlp_ms / 1e3) / 1e12
    if rank == 0:
        occ = []
        for sc in scs[:256]:
            k = np.floor(sc.y).astype(np.int64) * sc.size_x + np.floor(sc.x).astype(np.int64)
            occ.append(int(np.bincount(k).max()))
        line = {"metric": "particle-steps/s", "value": value, "unit": "particle-steps/s",
                "n_gpus": world, "steps": K, "warmup": W, "ms_per_step": L["ms"] / K,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32 state, bf16 network", "data": "synthetic",
                "config": {"workload": f"skewed ensemble, {len(scs)} scenes, {n} particles "
                                       f"(512-32,768 per scene, log-uniform), settled piles "
                                       f"({scenes.SETTLE_STEPS} plain steps) + 1-6 Gaussian blobs, "
                                       f"learned relaxation",
                           "particles": n, "cells": cells, "settle_s": t_settle,
                           "max_cell_occupancy_first_256": max(occ),
                           "parallelism": f"replicas x{world}", "launch_shapes": L["shapes"],
                           "long_row_masks": L["long_masks"]},
                "plain": {"value": world * n * K / (P["ms"] / 1e3), "ms_per_step": P["ms"] / K,
                          "kernel_ms": P["kernel_ms"], "clocks": P["clocks"]},
                "learned_vs_plain": P["ms"] / L["ms"],
                "rms_density_error_one_step": rms,
                "network_share_one_step": used / max(1, used + fell),
                "network_share_timed": (L["counts"][0] / max(1, sum(L["counts"]))),
                "threshold_rest_density": args.learned_threshold,
                "roofline": {"bound": "tensor", "kernel": "mlp", "achieved": achieved, "peak": peak,
                             "unit": "TFLOP/s", "frac": achieved / peak, "peak_source": peak_kind,
                             "flops_per_launch": MLP_FLOPS_PER_ROW * n},
                "kernel_ms": L["kernel_ms"], "clocks": L["clocks"], "gpu_launches": L["launches"],
                "training": info, "e2e": None, "cpu_baseline": None}
        print(json.dumps(line), flush=True)


def _gather_lists(counts, ids, owners):
    """Concatenated half lists of `owners` (ids into counts/ids as
    neighbor_lists returns them: counts by id, lists in id order)."""
    import numpy as np
    off = np.zeros(len(counts) + 1, np.int64)
    np.cumsum(counts, out=off[1:])
    lens = counts[owners].astype(np.int64)
    total = int(lens.sum())
    if total == 0:
        return np.zeros(0, ids.dtype)
    first = np.repeat(off[owners] - np.concatenate([[0], np.cumsum(lens)[:-1]]), lens)
    return ids[first + np.arange(total)]


def parity_window(sim, sc, params, cx0=560, cx1=640):
    """Parity of a full-size state against the oracle, on a window of it.
    The particles of grid columns [cx0, cx1) (the full height: the dense
    floor, the free surface, and the mover's path) are given, in id order,
    to the pinned CPU restatement of hash_fluid (hash.c:127-242) on the same
    grid; for the particles of columns [cx0 + 1, cx1 - 1), whose whole 3x3
    stencil lies in the window, the library's half lists over the WHOLE
    state must equal the oracle's (bit for bit, in the reference's order),
    their densities the reference's FP32 densities within 1e-5 relative per
    particle, and their relaxation displacements the FP64 gather oracle
    (fluid.c:541-611, from the library's densities) within 1e-5 of the
    summed magnitude of their pair terms."""
    import numpy as np

    import oracle
    t0 = time.perf_counter()
    st = sim.download()
    counts, ids = sim.neighbor_lists()
    rho, rhon = sim.probe_density(params)
    dx, dy = sim.probe_relaxation(params)
    x, y = st["x"], st["y"]
    with np.errstate(invalid="ignore"):
        cx = np.floor(x / np.float32(sc.spacing))
    win = np.nonzero((cx >= cx0) & (cx < cx1) & np.isfinite(y) & (y >= 0))[0]
    inner = (cx[win] >= cx0 + 1) & (cx[win] < cx1 - 1)
    z = np.zeros(len(win), np.float32)
    orc = oracle.Sim("port", x[win], y[win], z, z, params, sc.config())
    oc, oi = orc.hash(compute_density=True)
    ost = orc.get()
    loc = np.nonzero(inner)[0]
    g_own = win[loc]
    lists_ok = bool(np.array_equal(counts[g_own], oc[loc]) and
                    np.array_equal(_gather_lists(counts, ids, g_own),
                                   win[_gather_lists(oc, oi, loc)]))
    dens_err = 0.0
    dens_ok = True
    for got, want in ((rho[g_own], ost["density"][loc]), (rhon[g_own], ost["density_near"][loc])):
        got, want = got.astype(np.float64), want.astype(np.float64)
        d = np.abs(got - want)
        nz = want != 0
        dens_ok &= bool(np.all(d[~nz] == 0))
        dens_err = max(dens_err, float(np.max(d[nz] / np.abs(want[nz]), initial=0.0)))
    ox, oy, scale = orc.relax_f64(rho[win], rhon[win])
    orc.close()
    rel = 0.0
    relax_ok = True
    for got, want in ((dx[g_own], ox[loc]), (dy[g_own], oy[loc])):
        err = np.abs(got.astype(np.float64) - want)
        relax_ok &= bool(np.all(err <= 1e-5 * scale[loc] + 1e-9))
        rel = max(rel, float(np.max(err / (scale[loc] + 1e-30), initial=0.0)))
    return {"lists_bit_exact": lists_ok, "density_max_rel": dens_err,
            "density_ok": dens_ok and dens_err <= 1e-5,
            "relax_max_rel": rel, "relax_ok": relax_ok,
            "relax_tolerance": "|err| <= 1e-5 * sum |pair terms| + 1e-9 per component",
            "particles_checked": int(len(loc)), "window_particles": int(len(win)),
            "window": f"grid columns [{cx0 + 1}, {cx1 - 1}) of {sc.size_x}, full height",
            "half_list_entries_checked": int(counts[g_own].sum()),
            "seconds": time.perf_counter() - t0}


def run_gpu(args, world, rank):
    import numpy as np

    from sph_gb300 import scenes
    from sph_gb300.simulation import PinnedArray

    work = EnsembleWork(args.scenes) if args.workload == "ensemble" else DamBreak(args.n)
    n, cells = work.n, work.cells
    K, W = args.steps, args.warmup

    # ---- launch shapes: given, or tuned on a copy of the scene advanced to
    # the middle of the timed window (the gathers' costs drift as a scene
    # compresses), so that the timed steps are steps W .. W+K-1 of the run ----
    if args.shapes:
        given = [int(v) for v in args.shapes.split(",")]
        shapes, long_masks = given[:6], bool(given[6]) if len(given) > 6 else False
    else:
        tuner = work.fresh()
        work.advance(tuner, 0, W + K // 2)
        shapes = work.tune(tuner)
        long_masks = tuner.long_row_masks()
        tuner.close()

    # ---- device-resident throughput ----
    sim = work.fresh()
    sim.set_launch_shapes(shapes)
    sim.set_long_row_masks(long_masks)
    work.advance(sim, 0, W)
    t0 = W
    sim.synchronize()
    barrier(world)
    with ClockSampler(0) as clk:
        sim.timer_start()
        work.advance(sim, t0, K)
        ms = sim.timer_stop()
    clocks = clk.summary()
    ms = max_over_ranks(world, ms)
    barrier(world)
    value = world * n * K / (ms / 1e3)
    launches = sim.launches_per_step() * K
    diag = sim.diagnostics().tolist()
    counters = sim.counters()

    # ---- per-kernel times (CUDA events on the library stream) ----
    kt_runs = [sim.kernel_times(None) for _ in range(5)]
    ktimes = {k: statistics.median(r[k] for r in kt_runs) for k in kt_runs[0]}
    t_now = t0 + K + len(kt_runs)

    # ---- parity of this full-size state against the oracle (config 2) ----
    parity = None
    if args.workload == "dam_break" and not args.no_parity and rank == 0:
        try:
            parity = parity_window(sim, work.sc, work.p(t_now))
        except Exception as exc:  # reported, never hidden
            parity = {"error": f"{type(exc).__name__}: {exc}"}

    # ---- the same scene later in the run (compressed fluid) ----
    late = None
    if args.workload == "dam_break" and args.late_start > t_now and args.late_steps > 0:
        work.advance(sim, t_now, args.late_start - t_now)
        sim.synchronize()
        sim.timer_start()
        work.advance(sim, args.late_start, args.late_steps)
        ms_late = sim.timer_stop()
        late = {"steps_timed": f"{args.late_start}..{args.late_start + args.late_steps - 1}",
                "ms_per_step": ms_late / args.late_steps,
                "value": n * args.late_steps / (ms_late / 1e3),
                "step_frac": scenes.algorithmic_bytes_per_step(n, cells)
                / (ms_late / args.late_steps / 1e3) / 1e9 / load_peaks()[0]}
    sim.close()
    top = max(ktimes, key=ktimes.get)
    per_p, per_c = ALG_BYTES[top]
    alg = per_p * n + per_c * cells
    peak, peak_kind = load_peaks()
    achieved = alg / (ktimes[top] / 1e3) / 1e9
    step_bytes = scenes.algorithmic_bytes_per_step(n, cells)
    roofline = {"bound": "hbm", "kernel": top, "achieved": achieved, "peak": peak,
                "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
                "traffic": traffic_per_launch(top, n),
                "algorithmic_bytes_per_launch": alg,
                "step_algorithmic_bytes": step_bytes,
                "step_frac": step_bytes / (ms / K / 1e3) / 1e9 / peak,
                "kernel_ms": {k: round(v, 5) for k, v in ktimes.items()},
                "issue": issue_bound(top, n, ktimes[top], clocks.get("sm_mhz"))}

    # ---- end to end through the C ABI with host buffers ----
    e2e = None
    if not args.no_e2e:
        # two page-locked frames: the copy of frame t overlaps step t + 1,
        # and the host has every frame before the clock stops
        coords = [PinnedArray((n, 2), np.int16) for _ in range(2)]
        # the handle (device allocations, once per run like the reference's
        # own mallocs) and the initial state in page-locked host memory are
        # made before the clock starts; the upload from that memory is timed
        staged = []
        for a in work.state():
            pa = PinnedArray(a.shape, np.float32)
            pa.array[:] = a
            staged.append(pa)
        sim2 = work.blank()
        sim2.set_launch_shapes(shapes)
        sim2.set_long_row_masks(long_masks)
        sim2.synchronize()
        tw = time.perf_counter()
        sim2.upload(*[pa.array for pa in staged])
        for t in range(W + K):
            work.step_one(sim2, t)
            sim2.pack_coords_async(coords[t % 2].array)
            if t > 0:
                sim2.wait_coords(coords[(t - 1) % 2].array)
        sim2.wait_coords(coords[(W + K - 1) % 2].array)
        t_e2e = time.perf_counter() - tw
        sim2.close()
        state_bytes = sum(pa.array.nbytes for pa in staged)
        for c in coords + staged:
            c.free()
        t_e2e = max_over_ranks(world, t_e2e)
        e2e = {"value": world * n * (W + K) / t_e2e, "unit": "particle-steps/s",
               "h2d_bytes_per_step": int(work.tunables_bytes + state_bytes / (W + K)),
               "d2h_bytes_per_step": 4 * n,
               "steps": W + K, "includes": "state upload from page-locked host memory, then per "
                                           "step the tunables H2D, the full step and the packed "
                                           "coordinates D2H (pinned, double-buffered: frame t's "
                                           "copy overlaps step t+1); handle creation (device "
                                           "allocation) before the clock"}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = work.cpu_sample(args)

    learned = None
    if args.workload == "dam_break" and not args.no_learned:
        try:
            learned = run_learned(args, work, ms / K, shapes, long_masks)
        except Exception as exc:  # reported, never hidden
            learned = {"error": f"{type(exc).__name__}: {exc}"}

    if rank == 0:
        line = {"metric": "particle-steps/s", "value": value, "unit": "particle-steps/s",
                "n_gpus": world, "steps": K, "warmup": W, "ms_per_step": ms / K,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32", "data": "synthetic",
                "config": {"workload": work.name,
                           "particles": n, "cells": cells, "parallelism": f"replicas x{world}",
                           "l2": "no flush: per-step working set ~0.5 GB > 129 MB L2",
                           "steps_timed": f"{t0}..{t0 + K - 1}", "launch_shapes": shapes,
                           "long_row_masks": long_masks},
                "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu,
                "parity": parity, "late_window": late,
                "clocks": clocks, "gpu_launches": launches, "learned": learned,
                "diagnostics": {"mean_density": diag[0], "mean_near_density": diag[1],
                                "kinetic_energy_per_particle": diag[2]},
                "counters": counters}
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=480)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=4_194_304)
    ap.add_argument("--workload", default="dam_break", choices=["dam_break", "ensemble", "skewed"])
    ap.add_argument("--scenes", type=int, default=512)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-steps", type=int, default=12)
    ap.add_argument("--no-learned", action="store_true")
    ap.add_argument("--shapes", default="",
                    help="six ints: the gathers' launch shapes, and optionally a seventh, 1 for "
                         "long-row hit masks, instead of autotuning (profiling runs: under a "
                         "profiler the tuner's timings are not real)")
    ap.add_argument("--no-trajectory", action="store_true")
    ap.add_argument("--no-parity", action="store_true")
    ap.add_argument("--late-start", type=int, default=480,
                    help="a second timed window of --late-steps steps from this step of the run")
    ap.add_argument("--late-steps", type=int, default=20)
    ap.add_argument("--learned-threshold", type=float, default=0.01)
    ap.add_argument("--train-scenes", type=int, default=200)
    ap.add_argument("--train-n", type=int, default=65_536)
    ap.add_argument("--train-steps", type=int, default=300)
    ap.add_argument("--train-samples", type=int, default=6_000_000)
    ap.add_argument("--train-epochs", type=int, default=5)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    world, rank, _ = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
    elif args.workload == "skewed":
        if args.scenes == 512:
            args.scenes = 2048
        run_skewed(args, world, rank)
    else:
        run_gpu(args, world, rank)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
