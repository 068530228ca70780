"""GPU tests of the boundary's failure and asynchronous paths, through the C ABI:

  * the swarm kernel's one device wait (the barrier of the TMA bulk copy that
    stages a band) is bounded; the test hook lcf_set_wait_bound(0) makes every
    staged band's wait expire at once.  The fit must return LCF_E_TIMEOUT
    with no fault (each expiring warp lets its copy land, then stops taking
    tasks), and the context must stay usable: the next fit with the default
    bound is bit-identical to a fit that never saw the expiry;
  * lcf_fit_parametric_batch_async queues the fit and returns; lcf_wait with
    a short timeout reports LCF_E_TIMEOUT while it runs, other calls on the
    context are refused meanwhile, and the results once it completes equal
    the synchronous call's.
"""
import numpy as np
import pytest

from lightcurve_fitting_gb300 import abi, synth

pytestmark = pytest.mark.gpu

FIELDS = ["model", "rank", "pso_params", "pso_chi2", "svi_mu", "svi_log_sigma", "per_model_chi2", "mb_best_k",
          "mb_cost"]


@pytest.fixture(scope="module")
def ctx():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from lightcurve_fitting_gb300 import build
    build.build()
    from lightcurve_fitting_gb300.lib import Context
    c = Context(0)
    yield c
    c.close()


def _same(a, b):
    for name in FIELDS:
        x, y = getattr(a, name), getattr(b, name)
        ok = np.array_equal(x, y, equal_nan=True) if x.dtype.kind == "f" else np.array_equal(x, y)
        assert ok, name


def test_expired_device_wait_reports_timeout_and_the_context_recovers(ctx):
    from lightcurve_fitting_gb300.lib import LcfError
    batch = synth.config_uneven(12, seed=5)
    before = ctx.fit_batch(batch, fit_all_models=True, method=abi.METHOD_SVI)
    ctx.set_wait_bound(0)
    try:
        with pytest.raises(LcfError, match=f"status {abi.LCF_E_TIMEOUT}"):
            ctx.fit_batch(batch, fit_all_models=True, method=abi.METHOD_SVI)
    finally:
        ctx.set_wait_bound(1 << 24)
    after = ctx.fit_batch(batch, fit_all_models=True, method=abi.METHOD_SVI)
    _same(before, after)


def test_async_fit_and_bounded_wait(ctx):
    from lightcurve_fitting_gb300.lib import LcfError
    batch = synth.config_uneven(2000, seed=9)
    sync = ctx.fit_batch(batch, fit_all_models=True, method=abi.METHOD_SVI)
    res = ctx.fit_batch_async(batch, fit_all_models=True, method=abi.METHOD_SVI)
    # a 2,000-source fit runs for tens of milliseconds: a zero timeout finds it running
    assert ctx.wait(0) == abi.LCF_E_TIMEOUT
    with pytest.raises(LcfError, match="pending"):
        ctx.fit_batch(synth.config_uneven(2, seed=1))
    assert ctx.wait(-1) == 0
    _same(sync, res)
    assert ctx.wait(10) == 0  # nothing pending
    assert ctx.stats()["h2d_bytes"] > 0
