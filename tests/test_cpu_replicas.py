"""The benchmark's multi-GPU harness on the CPU: world size 2 over gloo.

One domain does not shard, so N GPUs run N independent replicas (each rank its own
scenario seed) and the step time is the maximum over ranks.  This runs bench.py's own
helpers in two processes over gloo on 127.0.0.1."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "WORLD_SIZE": str(world),
                       "RANK": str(rank), "LOCAL_RANK": str(rank), "LES_BENCH_GLOO": "1"})
    import numpy as np

    import bench
    import lesgpu
    w, r, local, pg = bench.dist_setup()
    t = bench.reduce_max(pg, 1.5 + r)                   # each rank's step time; the max is reported
    zbm = lesgpu.generate_scenario(bench.scenario(seed=1 + r, im=24, jm=16, km=10))[0]
    pg.barrier()
    out.put((r, w, t, float(np.asarray(zbm).sum())))
    pg.destroy_process_group()


def test_replicas_over_gloo():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, w0, t0, z0), (r1, w1, t1, z1) = res
    assert (r0, r1, w0, w1) == (0, 1, 2, 2)
    assert t0 == t1 == 2.5          # the maximum over ranks
    assert z0 != z1                 # each replica advances its own scenario
