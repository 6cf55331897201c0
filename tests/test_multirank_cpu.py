"""The multi-process path of bench.py on CPU: `--gpus N` runs N independent
replicas (one rank per GPU, the block per rank fixed: weak scaling), joined
only by a barrier around the timed region and a max over the ranks' times.
Two gloo ranks on 127.0.0.1 exercise those two helpers."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    bench.barrier(world)
    t = bench.max_over_ranks(10.0 * (rank + 1), world)   # rank r "took" 10 (r + 1) ms
    out.put((rank, t))
    bench.barrier(world)
    dist.destroy_process_group()


def test_replicas_take_the_slowest_rank():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = dict(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert res == {0: 20.0, 1: 20.0}
