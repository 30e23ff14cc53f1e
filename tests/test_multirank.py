"""The bench's multi-GPU host logic on two gloo ranks (CPU): every rank draws
its own batch (weak scaling, no exchange of pairs), the reported time is the
slowest rank's, and the value counts all ranks' pairs over that time."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import sys
    import torch
    import torch.distributed as dist
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    sys.path.insert(0, os.path.join(root, "mind-fcl_gb300"))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench
    from fclg import workloads
    dist.init_process_group("gloo", rank=rank, world_size=world)
    r, w, local = bench.dist_env()
    b = bench.rank_batch(workloads, "mixed", r, pairs=2000)
    fake_ms = 10.0 + 5.0 * r                     # rank 1 is the slow one
    ms = bench.max_over_ranks(torch, fake_ms, torch.device("cpu"), w)
    digest = float(np.sum(b.pairs["trans"]))
    out.put((r, w, local, ms, bench.job_value(b.n_pairs, w, ms), digest, b.n_pairs))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, w0, l0, ms0, v0, d0, n0), (r1, w1, l1, ms1, v1, d1, n1) = res
    assert (r0, r1) == (0, 1) and w0 == w1 == 2 and (l0, l1) == (0, 1)
    assert ms0 == ms1 == 15.0                    # max over ranks, the same everywhere
    assert v0 == v1 == 2 * 2000 / 15e-3          # all ranks' pairs over the slowest time
    assert n0 == n1 == 2000 and d0 != d1         # same batch shape, different draws
