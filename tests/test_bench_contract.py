"""Host-side checks of bench.py's bookkeeping against the library: the
per-kernel algorithmic bytes and the committed ncu traffic cover exactly the
kernels a step launches, and the canonical step budget is the one the
roofline fraction uses.  No call here touches a GPU."""
import json
import os

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
