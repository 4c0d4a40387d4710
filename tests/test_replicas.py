"""The multi-process path of bench.py on the CPU (world size 2, gloo): ranks
are independent replicas (a Bloch phase or a seed per rank), joined only by
a barrier and the max over ranks of their times; the reference arm runs on
rank 0 alone."""
import importlib
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    bench = importlib.import_module("bench")
    D = bench.Dist(world)
    D.barrier()
    m = D.max(float(10 * (rank + 1)))
    w, _, eps, _ = bench.setup_workload(1, rank)  # the 4x4x512 slab: cheap to build
    D.barrier()
    D.close()

    class A:
        workload, steps, warmup, cells = 1, 1, 1, 2
    ref = bench.run_reference(A, rank, world) if rank else "rank0"
    with open(os.path.join(out_dir, f"r{rank}.txt"), "w") as f:
        f.write(f"{m} {w.akx} {eps.shape} {ref}\n")


def test_two_gloo_ranks(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    r0 = open(tmp_path / "r0.txt").read().split(" ", 2)
    r1 = open(tmp_path / "r1.txt").read().split(" ", 2)
    assert float(r0[0]) == 20.0 and float(r1[0]) == 20.0  # max over ranks on both
    assert float(r1[1]) - float(r0[1]) == pytest.approx(0.01)  # each replica its own Bloch phase
    assert r1[2].strip().endswith("None")  # the reference arm prints on rank 0 only
