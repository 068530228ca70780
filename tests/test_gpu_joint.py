"""GPU tests of the joint multi-band Villar fit (fit_parametric with
fit_all_models = false and >= 2 bands, src/parametric.rs:3742-3761 and
fit_parametric_multiband :3815-4131), through the C ABI against the oracle.

The swarm is the reference's (200 particles, 1500 iterations, stall 60,
three seeds) in a 21-dimensional space for three bands; its FP32 cost
comparisons make its trajectory part from the FP64 oracle's, so two runs
end at different points of similar cost.  Checked:
  * the cost function itself: the joint cost the GPU reports equals the
    oracle's FP64 joint cost at the GPU's own best vector (1e-4 relative,
    the FP32 likelihood tolerance);
  * the dispatch and outputs: every fitted band is Villar with the oracle's
    rank, per-model chi2 holds Villar only and equals the joint cost;
  * the search: the GPU's joint costs are those of the oracle's search to
    5 % (median 1 %);
  * the reference's own multi-band test (tests/test_metal.rs:67-97).
"""
import numpy as np
import pytest

from lightcurve_fitting_gb300 import abi, synth

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


def _joint_vector(res, batch, s):
    bands = list(range(batch.source_band_offsets[s], batch.source_band_offsets[s + 1]))
    fitted = sorted([b for b in bands if res.rank[b] >= 0], key=lambda b: res.rank[b])
    ref = res.pso_params[fitted[0], :7]
    return np.concatenate([ref] + [res.pso_params[b, :7] - ref for b in fitted[1:]]), fitted


def test_joint_fit_matches_oracle(ctx, oracle):
    batch = synth.config_uneven(12, seed=5)
    g = ctx.fit_batch(batch, fit_all_models=False, method=abi.METHOD_LAPLACE, run_multi_bazin=False,
                      joint_multiband=True)
    r = oracle.fit_batch(batch, fit_all_models=False, method=abi.METHOD_LAPLACE, run_multi_bazin=False,
                         joint_multiband=True)
    assert np.array_equal(g.rank, r.rank)
    assert np.array_equal(g.model, r.model) and set(g.model[g.model >= 0]) == {1}
    fitted = g.model >= 0
    assert np.array_equal(g.per_model_chi2[fitted, 1], g.pso_chi2[fitted])
    assert np.isnan(np.delete(g.per_model_chi2[fitted], 1, axis=1)).all()
    rel_fn, rel_search = [], []
    for s in range(batch.n_sources):
        p, bands = _joint_vector(g, batch, s)
        c_gpu = g.pso_chi2[bands[0]]
        assert all(g.pso_chi2[b] == c_gpu for b in bands)
        c_orc_at_gpu = oracle.joint_cost(batch, s, p)
        rel_fn.append(abs(c_gpu - c_orc_at_gpu) / max(abs(c_orc_at_gpu), 1.0))
        c_orc = r.pso_chi2[bands[0]]
        rel_search.append((c_gpu - c_orc) / max(abs(c_orc), 1.0))
    assert max(rel_fn) < 1e-4, rel_fn
    assert max(np.abs(rel_search)) < 0.05 and np.median(np.abs(rel_search)) < 0.01, rel_search


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
