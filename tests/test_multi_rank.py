"""The multi-GPU host path of bench.py on CPU: world size 2 over gloo
(127.0.0.1).  Pairs are independent, so ranks only shard the work (each rank
its own seeded batch) and agree on the step time (max over ranks); there is
no collective on the data path."""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(ws), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    from alignment_projects_gb300 import synth
    w, r, local = bench.dist_env()
    dist = bench.dist_init(w, "gloo")
    t = bench.max_over_ranks(dist, 10.0 + r)            # step time: max over ranks
    bench.barrier(dist)
    batch = synth.montage_batch_torch(2 + 7919 * r, 2, "cpu", long_side=256)
    digest = float(sum(int(p["a"].sum()) + 3 * int(p["b"].sum()) for p in batch))
    q.put((r, t, digest))
    dist.destroy_process_group()


def test_two_ranks_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(k, 2, port, q)) for k in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    (r0, t0, d0), (r1, t1, d1) = out
    assert (r0, r1) == (0, 1)
    assert t0 == t1 == 11.0          # both ranks report the slowest rank's time
    assert d0 != d1                  # disjoint shards of the work
