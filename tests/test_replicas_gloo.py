"""The N > 1 path on CPU: world_size 2 over gloo.

bench.py runs one independent replica per rank (no data-path collective) and
reduces only the timing: a barrier on both sides of the timed region and the
max over ranks.  This checks that reduction and that replicas are independent
(each rank steps its own oracle state; results depend only on its own seed).
"""
import os
import socket

import numpy as np
import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from bench import reduce_time
    from oracle.pyoracle import OracleDyn, OracleSHT, set_threads
    from aeros_gb300.params import held_suarez_params
    set_threads(1)
    o = OracleDyn(held_suarez_params(trunc=5, nlev=4), nthreads=1)
    o.set_isothermal(264.0, 1e5)
    vor, div, t, lnps = o.get_state()
    rng = np.random.default_rng(1000 + rank)
    t = t.copy()
    t[:, 3] += rng.normal(0, 0.1, t.shape[0])
    o.set_state(vor, div, t, lnps)
    o.step(4)
    local = 0.001 * (rank + 1)
    tmax = reduce_time(local, world, backend="gloo")
    out.put((rank, tmax, o.get_state()[2].copy()))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_replicas():
    torch = pytest.importorskip("torch")
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = [q.get(timeout=120) for _ in range(2)]
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort(key=lambda r: r[0])
    assert res[0][1] == res[1][1] == pytest.approx(0.002)
    assert not np.array_equal(res[0][2], res[1][2])   # different seeds, independent replicas
