"""GPU tests of the joint multi-band Villar fit (fit_parametric with
fit_all_models = false and >= 2 bands, src/parametric.rs:3742-3761 and
fit_parametric_multiband :3815-4131), through the C ABI against the oracle.

The swarm is the reference's (200 particles, 1500 iterations, stall 60,
three seeds) in a 21-dimensional space for three bands, on the reference's
trajectory in double-float with FP32 cost comparisons (criteria.py states
the tolerances against the oracle's own sensitivity).  Checked:
  * the dispatch and outputs: every fitted band is Villar with the oracle's
    rank, per-model chi2 holds Villar only and equals the joint cost;
  * the cost function itself: the joint cost the GPU reports equals the
    oracle's FP64 joint cost at the GPU's own best vector (1e-6);
  * the search: the GPU's joint costs are the oracle's to a median 1e-6, with
    no more sources departing by 1e-4 than the oracle perturbed at 1e-6;
  * the reference's own multi-band test (tests/test_metal.rs:67-97).
"""
import numpy as np
import pytest

from lightcurve_fitting_gb300 import abi, synth

from criteria import check_joint

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


def test_joint_fit_matches_oracle(ctx, oracle):
    batch = synth.config_uneven(12, seed=5)
    kw = dict(fit_all_models=False, method=abi.METHOD_LAPLACE, run_multi_bazin=False, joint_multiband=True)
    check_joint(ctx.fit_batch(batch, **kw), oracle, batch, kw)


def test_joint_fit_on_basic_sources_matches_oracle(ctx, oracle):
    """40 basic sources (3 bands x 30 points): short bands, where the joint
    search is most sensitive."""
    batch = synth.config_basic(40, seed=21)
    kw = dict(fit_all_models=False, method=abi.METHOD_LAPLACE, run_multi_bazin=False, joint_multiband=True)
    check_joint(ctx.fit_batch(batch, **kw), oracle, batch, kw)


def test_reference_multiband_scenario(ctx, oracle):
    """tests/test_metal.rs:67-97 through the Python mirror: results for both
    bands, finite pso_chi2, model Villar."""
    from lightcurve_fitting_gb300 import parametric
    t = np.arange(30) * 1.5
    rf = oracle.eval_model(1, np.array([0.3, 0.01, 2.0, 10.0, 1.0, 3.0, -2.5]), t)
    e = np.abs(rf) * 0.05 + 0.01
    bands = {"ztfr": {"times": t, "values": rf, "errors": e},
             "ztfg": {"times": t, "values": 0.8 * rf, "errors": e}}
    res = parametric.fit_parametric(bands, False, "laplace", ctx=ctx)
    assert len(res) == 2
    for r in res:
        assert r["model"] == "Villar"
        assert r["pso_chi2"] is not None and np.isfinite(r["pso_chi2"])
        assert list(r["per_model_chi2"]) == ["Villar"]
    assert {r["band"] for r in res} == {"ztfr", "ztfg"}
