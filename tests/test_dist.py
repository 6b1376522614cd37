"""World-size-2 gloo test (CPU) of the multi-rank bench logic: one replica per rank, no
collective on the data path, a barrier around the timed region and the job time
taken as the maximum over ranks."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import bench
    r, w, local = bench.dist_env()
    dist = bench.init_dist(w, "gloo")
    bench.barrier(w)
    t = bench.reduce_max(10.0 + 5.0 * r, w)  # rank 1 is the slower replica
    # each replica processes its own seeded sub-integration; the job metric sums units over ranks
    units = 1000 * w
    q.put((r, w, local, t, units))
    bench.barrier(w)
    dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_two_rank_barrier_and_max():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=90) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1] and all(o[1] == 2 for o in out)
    assert all(o[3] == 15.0 for o in out)  # every rank sees the slowest rank's time


def test_single_rank_needs_no_process_group():
    import bench
    assert bench.reduce_max(3.5, 1) == 3.5
    bench.barrier(1)
