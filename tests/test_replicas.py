"""The multi-GPU form is replicas: under torchrun every rank advances its own
whole run, and bench.py takes the slowest rank's time and the sum of the
work.  This runs that coordination with two gloo ranks on the CPU, each
rank's replica being the C port of the step on its own seed."""
import os
import socket
import sys
import time

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    import oracle as O
    from qgw_gb300 import configs as C
    barrier, max_over_ranks = bench.rank_ops(world, "cpu")
    p = C.cfg1(32)
    q0 = C.noise_ic(p, 100 + rank)  # independent replicas
    barrier()
    t0 = time.perf_counter()
    r = O.run_port(p, q0, 5, dt_fixed=1200.0)
    dt = time.perf_counter() - t0 + 0.01 * rank  # ranks of different speed
    tmax = max_over_ranks(dt)
    value = bench.whole_job_rate(C.lgp(p), 5, tmax, world)
    out[rank] = (dt, tmax, value, float(np.abs(r["q"]).sum()))
    barrier()
    dist.destroy_process_group()


def test_two_replicas_over_gloo():
    world = 2
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_worker, args=(world, _free_port(), out), nprocs=world, join=True)
        res = dict(out)
    (d0, m0, v0, c0), (d1, m1, v1, c1) = res[0], res[1]
    assert m0 == m1 == max(d0, d1)  # every rank reports the slowest time
    assert v0 == v1 == pytest.approx(world * (31 * 31 * 3) * 5 / max(d0, d1))
    assert c0 != c1  # replicas ran different initial conditions
