"""The N > 1 host path of bench.py on CPU: two gloo ranks exercise the max-over-ranks timing
reduction, the barrier and the instance sharding of the batched workload (replicas / weak
scaling: no data-path collective)."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out_dir):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    r, w = bench.dist_env()
    assert (r, w) == (rank, world)
    # max over ranks of the per-rank timed region
    t = bench.reduce_max(10.0 + rank, w)
    bench.barrier(w)
    # the batched workload takes instances rank*n .. rank*n + n - 1
    n = 3
    specs = [bench.batch_spec(rank * n + i) for i in range(n)]
    with open(os.path.join(out_dir, f"rank{rank}.txt"), "w") as f:
        f.write(f"{t}\n")
        for m, p, th, amps in specs:
            f.write(f"{m} {p} {th:.12g} {' '.join(f'{a:.12g}' for a in amps)}\n")
    dist.destroy_process_group()


def test_two_gloo_ranks(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    port = _free_port()
    mp.spawn(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    lines = [open(tmp_path / f"rank{r}.txt").read().splitlines() for r in range(2)]
    # both ranks see the maximum of their timings
    assert float(lines[0][0]) == 11.0 and float(lines[1][0]) == 11.0
    # disjoint instance shards, each equal to the single-process specification of those indices
    sys.path.insert(0, ROOT)
    import bench
    assert lines[0][1:] != lines[1][1:]
    for r in range(2):
        for i, line in enumerate(lines[r][1:]):
            m, p, th, amps = bench.batch_spec(r * 3 + i)
            assert line.split()[:2] == [str(m), str(p)]
