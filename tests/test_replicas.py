"""The multi-GPU replica path of bench.py on CPU: two gloo ranks (no GPU).

Instances are independent, so each rank steps its own ensemble -- the same
size mix with seeds of its own -- and the only collective is the max of the
timed windows; the job's rate counts every rank's instances against the
slowest rank's time."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        specs = bench.rank_specs(8, 1234, rank)
        ms = bench.max_over_ranks(10.0 + rank, dist, "cpu")      # rank 1 is the slower one
        out.put((rank, [(s["n_r_max"], s["m_max"], s["ra"], s["seed"]) for s in specs], ms,
                 bench.aggregate_rate(world, len(specs), 5, ms)))
    finally:
        dist.destroy_process_group()


def test_two_gloo_replicas():
    import multiprocessing as mp
    import socket
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, s0, ms0, v0), (r1, s1, ms1, v1) = res
    assert (r0, r1) == (0, 1)
    assert ms0 == ms1 == 11.0                       # the slower rank's window on both
    assert v0 == v1 == 2 * 8 * 5 / 11.0e-3          # both ranks' instances against it
    assert [x[3] for x in s0] != [x[3] for x in s1]  # seeds of their own
    assert sorted((a, b) for a, b, _, _ in s0) != [] and all(a in (33, 49, 65) for a, _, _, _ in s0 + s1)

