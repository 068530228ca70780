"""The MultiBazin branch (lcf_set_multi_bazin_branch): K = 2..4 of the
greedy MultiBazin loop on a second stream, forked from the stage sequence
after the model-selection swarms or after the selection, must give the same
results as the stages run in sequence, with and without the captured graph."""
import numpy as np
import pytest

from lightcurve_fitting_gb300 import abi, synth

pytestmark = pytest.mark.gpu

FIELDS = ["model", "rank", "pso_params", "pso_chi2", "svi_mu", "svi_log_sigma", "svi_elbo", "mag_chi2",
          "per_model_chi2", "per_model_params", "mb_best_k", "mb_params", "mb_cost", "mb_bic", "mb_per_k_cost",
          "mb_per_k_bic"]


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
    c.set_multi_bazin_branch(1)
    c.set_graph(True)
    c.close()


def _same(a, b):
    return np.array_equal(a, b, equal_nan=True) if a.dtype.kind == "f" else np.array_equal(a, b)


@pytest.mark.parametrize("fit_all", [True, False])
def test_branch_modes_give_identical_results(ctx, fit_all):
    batch = synth.config_uneven(40, seed=71)
    runs = {}
    for graph in (True, False):
        ctx.set_graph(graph)
        for mode in (0, 1, 2):
            ctx.set_multi_bazin_branch(mode)
            runs[(graph, mode)] = ctx.fit_batch(batch, fit_all_models=fit_all, method=abi.METHOD_SVI)
            st = ctx.stats()
            assert st["ms_multi_bazin"] > 0.0 and st["ms_total"] > 0.0
    base = runs[(True, 0)]
    assert np.sum(base.mb_best_k > 0) >= 30
    for key, r in runs.items():
        for name in FIELDS:
            assert _same(getattr(r, name), getattr(base, name)), (key, name)


def test_branch_mode_is_checked(ctx):
    from lightcurve_fitting_gb300.lib import LcfError
    with pytest.raises(LcfError):
        ctx.set_multi_bazin_branch(3)


def test_branch_timing_survives_other_entry_points(ctx):
    """A graph replay after a finalisation call still times the branch."""
    ctx.set_graph(True)
    ctx.set_multi_bazin_branch(1)
    batch = synth.config_basic(8, seed=73)
    r = ctx.fit_batch(batch, fit_all_models=True, method=abi.METHOD_LAPLACE)
    ctx.finalize_batch(batch, r.model, r.pso_params, method=abi.METHOD_LAPLACE)
    assert ctx.stats()["ms_multi_bazin"] == 0.0
    ctx.fit_batch(batch, fit_all_models=True, method=abi.METHOD_LAPLACE)
    assert ctx.stats()["ms_multi_bazin"] > 0.0
