"""The multi-GPU form of bench.py is N independent replicas (the step does
not shard on one device); torchrun ranks only share a barrier and the
max-over-ranks time.  Checked here on CPU with gloo, world size 2."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    sys.path.insert(0, ROOT)
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import bench
    w, r, local = bench.dist_setup()
    assert (w, r, local) == (world, rank, rank)
    # each rank sees exactly one device: its own
    assert os.environ["CUDA_VISIBLE_DEVICES"] == str(rank)
    bench.barrier(w)
    t = bench.max_over_ranks(w, 10.0 + rank)
    out[rank] = t
    import torch.distributed as dist
    dist.destroy_process_group()


def test_max_over_ranks_gloo():
    port = _free_port()
    out = mp.Manager().dict()
    os.environ.pop("CUDA_VISIBLE_DEVICES", None)
    mp.spawn(_rank_main, args=(2, port, out), nprocs=2, join=True)
    assert dict(out) == {0: 11.0, 1: 11.0}


def test_reference_arm_prints_on_rank0_only(capsys):
    sys.path.insert(0, ROOT)
    import bench

    class A:
        n, steps, warmup, gpus = 16384, 2, 3, 2
    bench.run_reference(A, world=2, rank=1)
    assert capsys.readouterr().out == ""
