"""The swarm launch autotuner (lcf_set_autotune / lcf_autotune_* in
include/lcf.h): every candidate launch shape and staging depth gives
bit-identical fits, the online tuner explores each candidate once per shape
bucket and then keeps the fastest, and an exported table preloads a new
context."""
import numpy as np
import pytest

from lightcurve_fitting_gb300 import abi, synth

pytestmark = pytest.mark.gpu

FIELDS = ["model", "rank", "pso_params", "pso_chi2", "svi_mu", "svi_log_sigma", "svi_elbo", "mag_chi2",
          "per_model_chi2", "per_model_params", "mb_best_k", "mb_params", "mb_cost"]


@pytest.fixture(scope="module")
def lib():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from lightcurve_fitting_gb300 import build
    build.build()
    from lightcurve_fitting_gb300 import lib as L
    return L


def _same(a, b):
    for name in FIELDS:
        x, y = getattr(a, name), getattr(b, name)
        ok = np.array_equal(x, y, equal_nan=True) if x.dtype.kind == "f" else np.array_equal(x, y)
        if not ok:
            return name
    return None


@pytest.mark.parametrize("workload", ["uneven", "long"])
def test_every_candidate_gives_identical_fits(lib, workload):
    # long: bands of 240-1,920 points, so the three staging depths (256, 512,
    # 1,024 observations) stage different bands in shared memory
    batch = synth.config_uneven(24, seed=41) if workload == "uneven" else synth.config_precision(3, seed=4)
    ctx = lib.Context(0)
    try:
        cands = ctx.autotune_candidates()
        assert cands.shape == (3, 3) and np.all(cands[:, 2] >= 1)
        res = []
        for c in range(cands.shape[0]):
            ctx.set_autotune(1, c)
            res.append(ctx.fit_batch(batch, fit_all_models=True, method=abi.METHOD_SVI))
            assert ctx.last_launch()["candidate"] == c
        for c in range(1, len(res)):
            assert _same(res[0], res[c]) is None, (c, _same(res[0], res[c]))
    finally:
        ctx.close()


def test_online_tuning_explores_then_keeps_the_fastest(lib):
    batch = synth.config_uneven(40, seed=43)
    ctx = lib.Context(0)
    try:
        first = None
        for k in range(3):
            r = ctx.fit_batch(batch, fit_all_models=True, method=abi.METHOD_SVI)
            assert ctx.last_launch()["candidate"] == k
            first = first or r
            assert _same(first, r) is None
        table = ctx.autotune_table()
        assert table.shape == (1, 6)
        bucket, best, nxt = int(table[0, 0]), int(table[0, 1]), int(table[0, 2])
        assert nxt == 3 and best == int(np.argmin(table[0, 3:])) and np.all(table[0, 3:] > 0)
        r = ctx.fit_batch(batch, fit_all_models=True, method=abi.METHOD_SVI)
        last = ctx.last_launch()
        assert last["candidate"] == best and last["bucket"] == bucket
        assert _same(first, r) is None
        # a batch of another shape gets its own bucket
        ctx.fit_batch(synth.config_uneven(300, seed=44), fit_all_models=True, method=abi.METHOD_SVI)
        assert ctx.autotune_table().shape[0] == 2 and ctx.last_launch()["candidate"] == 0
    finally:
        ctx.close()
    # the table preloads a new context: no exploration for that bucket
    ctx2 = lib.Context(0)
    try:
        ctx2.autotune_load(table)
        ctx2.fit_batch(batch, fit_all_models=True, method=abi.METHOD_SVI)
        assert ctx2.last_launch()["candidate"] == best
        ctx2.set_autotune(0)
        ctx2.fit_batch(batch, fit_all_models=True, method=abi.METHOD_SVI)
        assert ctx2.last_launch()["candidate"] == 0
    finally:
        ctx2.close()
