"""Multi-GPU form: independent replicas (the step does not shard), exercised here as two gloo
ranks on the CPU with the oracle's restatement standing in for the per-rank model.

Each rank advances its own member (seed = rank); the ranks agree on the slowest time with an
all-reduce MAX, as bench.py does over NCCL, and no state is exchanged."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as tmp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import time
    import torch
    from epic_gb300 import EPIC_SYNC_DIAGS_ONLY, HSConfig, hs_setup
    from oracle_lib import Port
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ga, f = hs_setup(HSConfig(ni=32, nj=16, nk=10, dt=300, seed=rank))
    p = Port(ga)
    p.upload(f)
    p.timestep(EPIC_SYNC_DIAGS_ONLY)
    dist.barrier()
    t0 = time.perf_counter()
    p.run(3)
    t = torch.tensor([time.perf_counter() - t0])
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    out[rank] = (float(t.item()), p.download().theta.copy())
    dist.destroy_process_group()


def test_two_rank_replicas_are_independent():
    port = _free_port()
    mgr = tmp.Manager()
    out = mgr.dict()
    tmp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
    t0, th0 = out[0]
    t1, th1 = out[1]
    assert t0 == t1 > 0          # both ranks report the max over ranks
    assert not np.array_equal(th0, th1)   # different seeds, different members
    # rank 1's member equals the same member stepped alone
    import sys
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from epic_gb300 import EPIC_SYNC_DIAGS_ONLY, HSConfig, hs_setup
    from oracle_lib import Port
    ga, f = hs_setup(HSConfig(ni=32, nj=16, nk=10, dt=300, seed=1))
    p = Port(ga)
    p.upload(f)
    p.timestep(EPIC_SYNC_DIAGS_ONLY)
    p.run(3)
    assert np.array_equal(p.download().theta, th1)
