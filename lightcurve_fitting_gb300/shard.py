"""Sharding of one batch across processes / GPUs, and the gather of their results.

Every source is fitted independently (fit_parametric_model runs per band, the
MultiBazin fit per source), so a batch splits into shards with no exchange on
the data path: each rank fits its own sources, and the only communication is
the host gather of the per-band results back into the caller's source order.

The shards are balanced by estimated work.  A source's swarm work is its
observation count times the particle evaluations per observation,
models x restarts x particles (8 x 3 x 30, src/parametric.rs:1974-2011): the
sources are taken longest first and each goes to the rank with the least work
so far (greedy longest-processing-time), so the shards' lengths stay within one
source's work of each other however uneven the band lengths are.
"""
from __future__ import annotations

import numpy as np

from . import abi

# particle evaluations per observation of a source in model selection:
# 8 models x 3 restarts x 30 particles (each evaluated ~61 times per run)
EVALS_PER_OBS = 8 * 3 * 30


def source_work(batch) -> np.ndarray:
    """Estimated swarm work per source: observations x models x restarts x particles."""
    obs = np.asarray(batch.band_obs_offsets, np.int64)
    sbo = np.asarray(batch.source_band_offsets, np.int64)
    n_per_source = obs[sbo[1:]] - obs[sbo[:-1]]
    return n_per_source.astype(np.float64) * EVALS_PER_OBS


def partition(batch, n_ranks: int) -> list:
    """The sources of each rank: greedy longest-processing-time over
    source_work, ties broken by source index; each rank's list ascending."""
    if n_ranks < 1:
        raise ValueError("n_ranks must be >= 1")
    work = source_work(batch)
    order = np.lexsort((np.arange(work.size), -work))
    load = np.zeros(n_ranks)
    owner = np.empty(work.size, np.int64)
    for s in order:
        r = int(np.argmin(load))
        owner[s] = r
        load[r] += work[s]
    return [np.flatnonzero(owner == r) for r in range(n_ranks)]


def gather(batch, parts: list, results: list) -> abi.FitResult:
    """One FitResult in the caller's band order from the ranks' results
    (results[r] fitted batch.subset(parts[r]))."""
    out = abi.FitResult(batch.n_bands)
    names = [k for k in vars(out) if k != "n_bands"]
    sbo = batch.source_band_offsets
    for srcs, res in zip(parts, results):
        srcs = np.asarray(srcs, np.int64)
        cnt = (sbo[srcs + 1] - sbo[srcs]).astype(np.int64)
        # global band indices of the shard's bands, in the shard's order
        glob = np.repeat(sbo[srcs].astype(np.int64), cnt) + (np.arange(int(cnt.sum())) -
                                                            np.repeat(np.cumsum(cnt) - cnt, cnt))
        if glob.size != res.n_bands:
            raise ValueError("a shard's result does not match its sources")
        for k in names:
            getattr(out, k)[glob] = getattr(res, k)
    return out
