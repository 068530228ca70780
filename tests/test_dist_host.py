"""Multi-rank host logic of bench.py on CPU: two `gloo` ranks (spawned
processes) take their own shards of the uneven workload (no exchange on the
data path), agree on the slowest rank's step time through the same
all-reduce the GPU run uses, and report the whole-job value from it."""
import multiprocessing as mp
import os
import socket

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, ws, port, q):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist
    import bench
    try:
        w, r, local = bench.dist_setup()
        shard = bench.rank_workload(40, r)
        step_ms = 100.0 + 25.0 * r  # this rank's step time
        mx = bench.dist_max(step_ms, w, "cpu")
        bench.dist_barrier(w)
        q.put((r, w, mx, shard.n_sources, shard.n_bands, float(np.sum(shard.flux)),
               bench.job_value(shard.n_sources, w, mx)))
    finally:
        if dist.is_initialized():
            dist.destroy_process_group()


def test_two_gloo_ranks_shard_and_take_the_max():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    (r0, w0, mx0, ns0, nb0, fs0, v0), (r1, w1, mx1, ns1, nb1, fs1, v1) = out
    assert (r0, r1, w0, w1) == (0, 1, 2, 2)
    assert mx0 == mx1 == 125.0                    # the slowest rank's time
    assert ns0 == ns1 == 40 and nb0 == nb1 == 120  # equal work per rank (weak scaling)
    assert fs0 != fs1                              # independent shards
    assert v0 == v1 == 2 * 40 / 0.125              # all ranks' sources / max time
