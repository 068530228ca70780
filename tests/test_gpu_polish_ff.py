"""GPU tests of the polish's double-float observation term (models_ff.cuh)
against its FP64 term (models_f64.cuh), through lcf_probe_ff: the cost,
gradient and upper-limit terms of PsoCost::cost_from_slice /
PsoCost::gradient (src/parametric.rs:1303-1446) at 256 points of each
model's PSO box over a band with 27 % upper limits.

Tolerances, relative to the sum of the terms' magnitudes:
  * cost: 1e-12, except Afterglow (1e-8), whose ln(ps) amplifies the
    reference's own rounding of ln(1 + e^ph) (FP64 forms 1 + e^ph before the
    logarithm; double-float keeps the small e^ph);
  * gradient (detections): 1e-5, the reference's own cancellation in
    1 - sigma(x) of the rise sigmoids (double-float forms 1 - sigma from
    e^-|x|); elsewhere the two agree to ~1e-12.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


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


def test_ff_term_matches_fp64_term(ctx):
    r = ctx.probe_ff()
    by = np.array(r["worst_rel_by_component"])  # [model][cost, g0..g6]
    cost_tol = np.array([1e-12] * 6 + [1e-8])
    assert np.all(by[:, 0] < cost_tol), by[:, 0]
    assert np.all(by[:, 1:] < 1e-5), by[:, 1:]
    assert r["nonfinite_mismatch"] == 0
    # most of each box runs in double-float (the rest falls back to FP64)
    assert min(r["points_in_range"]) >= 100, r["points_in_range"]


def test_ff_term_outpaces_fp64_term(ctx):
    ff = np.array(ctx.probe_ff()["obs_evals_per_s"])
    f64 = np.array(ctx.probe_fp64()["obs_evals_per_s"][:7])
    assert np.all(ff > 2.0 * f64), (ff, f64)


def test_polish_runs_in_double_float(ctx):
    """On the synthetic workload nearly every polish evaluation stays in
    double-float; the counters split the work by arithmetic."""
    from lightcurve_fitting_gb300 import abi, synth
    batch = synth.config_uneven(60, seed=3)
    ctx.fit_batch(batch, fit_all_models=True, method=abi.METHOD_SVI)
    st = ctx.stats()
    tot = sum(st["lbfgs_obs_evals_by_model"][:7])
    fb = sum(st["lbfgs_fp64_obs_evals_by_model"][:7])
    assert tot > 0 and fb <= 0.05 * tot, (fb, tot)
