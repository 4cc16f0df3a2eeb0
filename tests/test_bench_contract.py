"""Host-side checks of bench.py's bookkeeping against the library: the
per-kernel algorithmic bytes and the committed ncu traffic cover exactly the
kernels a step launches, and the canonical step budget is the one the
roofline fraction uses.  No call here touches a GPU."""
import json
import os

import numpy as np

import bench
from sph_gb300 import scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def step_kernel_names(lib):
    names = []
    for k in range(16):
        s = lib.sph_cuda_step_kernel_name(None, k)
        if not s:
            break
        names.append(s.decode())
    return names


def test_alg_bytes_cover_the_step_kernels(cuda_lib):
    names = step_kernel_names(cuda_lib)
    assert len(names) == 9
    assert sorted(bench.ALG_BYTES) == sorted(names)


def test_traffic_capture_covers_the_step_kernels(cuda_lib):
    with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
        t = json.load(f)
    names = step_kernel_names(cuda_lib)
    assert sorted(t["kernels"]) == sorted(names)
    for k, v in t["kernels"].items():
        assert v["dram_bytes"] == v["dram_read"] + v["dram_write"], k
        assert v["dram_bytes"] > 0, k
    n = t["particles"]
    assert bench.traffic_per_launch("viscosity_predict", n) == t["kernels"]["viscosity_predict"]["dram_bytes"]
    assert bench.traffic_per_launch("viscosity_predict", 2 * n) == 2 * t["kernels"]["viscosity_predict"]["dram_bytes"]


def test_canonical_step_bytes():
    sc = scenes.config2()
    assert scenes.algorithmic_bytes_per_step(sc.n, sc.cells) == 216 * 4_194_304 + 16 * 6_444_050 == 1_009_074_464


def test_slab_partition_is_the_references():
    """partitionProblem (geometry.c:101-160): floor(columns / ranks) columns
    each, the remainder to the leftmost ranks; the slabs cover every
    particle exactly once."""
    assert scenes.slab_columns(2393, 16)[:10] == [(150 * i, 150) for i in range(9)] + [(1350, 149)]
    assert scenes.slab_columns(2393, 16)[-1] == (2244, 149)
    sc = scenes.config2(n=65536)
    parts = [scenes.slab_indices(sc, s, 8) for s in range(8)]
    allidx = np.sort(np.concatenate(parts))
    assert np.array_equal(allidx, np.arange(sc.n))
    assert min(len(p) for p in parts) > 0


def test_reference_arm_prints_the_contract_line(tmp_path):
    """`bench.py --impl reference` on a small dam break: one JSON line with
    the reference arm's keys (it runs the CPU step only, no GPU), on the
    steps it was asked for."""
    import subprocess
    import sys
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                          "--n", "16384", "--steps", "2", "--warmup", "3"],
                         capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == "particle-steps/s" and d["value"] > 0
    assert d["higher_is_better"] is True and d["unit"] == "particle-steps/s"
    assert d["cpu_baseline"]["value"] == d["value"] and d["cpu_baseline"]["cores"] >= 1
    assert d["cpu_baseline"]["kind"] in ("port", "reference")
    assert d["e2e"] == {"value": d["value"], "unit": "particle-steps/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
    assert d["steps"] == 2 and d["warmup"] == 3 and d["config"]["particles"] == 16384
