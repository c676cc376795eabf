"""Multi-GPU path of the bench on CPU: two gloo ranks.

The path shards by disorder sample with no data-path collective: rank r
solves samples [r * 100, (r + 1) * 100) of every class, and the ranks meet
only to report the slowest rank's time and the total count.
"""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    samples = sorted({p.sample for p in bench.problems(rank)})
    classes = sorted({p.error_class for p in bench.problems(rank)})
    times, counts = bench.reduce_over_ranks(dist, [1.0 + rank, 10.0 - rank, 0.5 * rank], [100 + rank, 7], "cpu")
    dist.destroy_process_group()
    q.put((rank, samples, classes, times, counts))


def test_two_ranks_shard_disjoint_samples_and_reduce():
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = dict((r, rest) for r, *rest in (q.get(timeout=120) for _ in procs))
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    s0, s1 = set(out[0][0]), set(out[1][0])
    assert s0 == set(range(100)) and s1 == set(range(100, 200))
    assert out[0][1] == out[1][1] == [b"c", b"h", b"i", b"v"]
    for r in (0, 1):
        times, counts = out[r][2], out[r][3]
        assert times == [2.0, 10.0, 0.5]      # max over ranks
        assert counts == [201, 14]            # sum over ranks
