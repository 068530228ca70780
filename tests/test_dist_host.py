"""Multi-rank host logic on CPU, with two `gloo` ranks in spawned processes:

  * bench.py's shards: every rank builds the same workload and takes its
    partition (lightcurve_fitting_gb300.shard: greedy by estimated work), the
    ranks agree on the slowest rank's step time through the same all-reduce
    the GPU run uses, and report the whole-job value from it;
  * partition -> fit -> gather: each rank fits its shard (with the oracle, so
    that no GPU is needed), rank 0 gathers the results and reassembles them in
    the caller's source order, bit-identical to a single-process fit of all
    the sources.
"""
import multiprocessing as mp
import os
import socket

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _env(rank, ws, port):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))


def _bench_worker(rank, ws, port, q):
    import sys
    sys.path.insert(0, ROOT)
    _env(rank, ws, port)
    import torch.distributed as dist
    import bench
    try:
        w, r, local = bench.dist_setup()
        shard = bench.rank_workload(40, r, w)
        step_ms = 100.0 + 25.0 * r  # this rank's step time
        mx = bench.dist_max(step_ms, w, "cpu")
        bench.dist_barrier(w)
        q.put((r, w, mx, shard.n_sources, int(shard.n_obs), bench.job_value(40, w, mx)))
    finally:
        if dist.is_initialized():
            dist.destroy_process_group()


def _run(target, ws, *args):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=target, args=(r, ws, port, q) + args) for r in range(ws)]
    for p in procs:
        p.start()
    out = [q.get(timeout=300) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    return sorted(out, key=lambda x: x[0])


def test_two_gloo_ranks_partition_one_workload_and_take_the_max():
    import sys
    sys.path.insert(0, ROOT)
    from lightcurve_fitting_gb300 import shard, synth
    out = _run(_bench_worker, 2)
    (r0, w0, mx0, ns0, no0, v0), (r1, w1, mx1, ns1, no1, v1) = out
    assert (r0, r1, w0, w1) == (0, 1, 2, 2)
    assert mx0 == mx1 == 125.0                 # the slowest rank's time
    assert ns0 + ns1 == 80                     # one workload of 2 x 40 sources, split
    full = synth.config_uneven(80, seed=2)
    assert no0 + no1 == full.n_obs
    # balanced by work: within the largest source's work of each other
    w = shard.source_work(full)
    assert abs(no0 - no1) * shard.EVALS_PER_OBS <= w.max()
    assert v0 == v1 == 2 * 40 / 0.125          # all ranks' sources / max time


def _fit_worker(rank, ws, port, q):
    import sys
    sys.path.insert(0, ROOT)
    _env(rank, ws, port)
    import torch.distributed as dist
    from lightcurve_fitting_gb300 import abi, shard, synth
    from oracle import oracle as O
    dist.init_process_group("gloo")
    try:
        batch = synth.config_uneven(10, seed=7)
        parts = shard.partition(batch, ws)
        res = O.fit_batch(batch.subset(parts[rank]), fit_all_models=True, method=abi.METHOD_SVI,
                          run_multi_bazin=True, n_threads=1)
        got = [None] * ws if rank == 0 else None
        dist.gather_object(res, got, dst=0)
        if rank == 0:
            q.put((rank, shard.gather(batch, parts, got), [p.tolist() for p in parts]))
        else:
            q.put((rank, None, None))
    finally:
        dist.destroy_process_group()


def test_partition_fit_gather_equals_a_single_process_fit():
    import sys
    sys.path.insert(0, ROOT)
    from lightcurve_fitting_gb300 import abi, synth
    from oracle import oracle as O
    O.build()
    out = _run(_fit_worker, 2)
    gathered, parts = out[0][1], out[0][2]
    assert sorted(parts[0] + parts[1]) == list(range(10)) and parts[0] and parts[1]
    batch = synth.config_uneven(10, seed=7)
    single = O.fit_batch(batch, fit_all_models=True, method=abi.METHOD_SVI, run_multi_bazin=True, n_threads=1)
    for k in vars(single):
        if k == "n_bands":
            continue
        a, b = getattr(gathered, k), getattr(single, k)
        assert np.array_equal(a, b, equal_nan=True) if a.dtype.kind == "f" else np.array_equal(a, b), k
