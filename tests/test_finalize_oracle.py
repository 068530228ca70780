"""CPU tests of the batched finalisation restatement (oracle/lcf_oracle.cpp
finalize_source: finalize_parametric_from_gpu, finalize_parametric_with_gpu_svi
and finalize_all_models_with_gpu_svi, src/parametric.rs:3126-3553).

The three reference functions run the tail of fit_parametric_model
(:3563-3739) from an externally selected model and PSO parameters, so the
oracle's finalisation fed with the oracle's own selection must reproduce the
oracle's full fit exactly.
"""
import numpy as np
import pytest

from lightcurve_fitting_gb300 import abi, synth

FIELDS = ["model", "rank", "n_obs", "pso_params", "pso_chi2", "svi_mu", "svi_log_sigma", "svi_elbo", "mag_chi2",
          "per_model_chi2"]


def _same(a, b):
    return np.array_equal(a, b, equal_nan=True) if a.dtype.kind == "f" else np.array_equal(a, b)


@pytest.mark.parametrize("method", [abi.METHOD_LAPLACE, abi.METHOD_SVI])
def test_finalize_from_own_selection_reproduces_the_fit(oracle, method):
    """finalize_parametric_from_gpu: uncertainty from the selection's PSO
    parameters (after the profile t0 search, which the fit reports), then the
    refinements and the magnitude chi2: bit-identical to the full fit."""
    batch = synth.config_basic(4, seed=31)
    ref = oracle.fit_batch(batch, fit_all_models=True, method=method, run_multi_bazin=False)
    fin = oracle.finalize_batch(batch, ref.model, ref.pso_params, ref.pso_chi2, ref.per_model_chi2, method=method)
    for name in FIELDS:
        assert _same(getattr(fin, name), getattr(ref, name)), name
    assert np.all(np.isnan(fin.per_model_params)) and np.all(fin.mb_best_k == 0)


def test_finalize_with_given_svi_outputs(oracle):
    """finalize_*_with_gpu_svi: the supplied (mu, log sigma, elbo) replace the
    uncertainty stage.  Supplying the oracle's own svi_fit outputs gives the
    finalize_parametric_from_gpu result exactly."""
    batch = synth.config_basic(3, seed=37)
    ref = oracle.fit_batch(batch, fit_all_models=True, method=abi.METHOD_SVI, run_multi_bazin=False)
    nb = batch.n_bands
    mu = np.full((nb, 7), np.nan)
    ls = np.full((nb, 7), np.nan)
    elbo = np.full(nb, np.nan)
    for s in range(batch.n_sources):
        for k, (t, f, e) in enumerate(batch.bands_of(s)):
            b = batch.source_band_offsets[s] + k
            m = int(ref.model[b])
            if m < 0:
                continue
            n = abi.N_PARAMS[m]
            u_mu, u_ls, u_elbo, _ = oracle.svi_fit(m, _band(oracle, t, f, e), ref.pso_params[b, :n])
            mu[b, :n], ls[b, :n], elbo[b] = u_mu, u_ls, u_elbo
    given = oracle.finalize_batch(batch, ref.model, ref.pso_params, ref.pso_chi2, ref.per_model_chi2, mu, ls, elbo)
    for name in FIELDS:
        assert _same(getattr(given, name), getattr(ref, name)), name


def _band(oracle, t, f, e):
    return oracle.Band(t, f, e)


def test_finalize_skips_unselected_and_unfittable_bands(oracle):
    """model -1 (an empty pso_params in the reference) and a band the
    preparation rejects (peak flux <= 0) both come back unfitted; the others
    keep their by-count rank."""
    batch = synth.config_basic(2, seed=41)
    ref = oracle.fit_batch(batch, fit_all_models=True, method=abi.METHOD_LAPLACE, run_multi_bazin=False)
    model = ref.model.copy()
    model[0] = -1
    o0, o1 = batch.band_obs_offsets[4], batch.band_obs_offsets[5]
    batch.flux[o0:o1] = -np.abs(batch.flux[o0:o1])
    fin = oracle.finalize_batch(batch, model, ref.pso_params, method=abi.METHOD_LAPLACE)
    assert fin.model[0] == -1 and fin.rank[0] == -1
    assert fin.model[4] == -1 and fin.rank[4] == -1
    keep = [b for b in range(batch.n_bands) if b not in (0, 4)]
    assert np.all(fin.model[keep] == ref.model[keep])
    assert np.all(np.isnan(fin.pso_chi2)) and np.all(np.isnan(fin.per_model_chi2))


def test_selection_struct_checks_shapes():
    with pytest.raises(ValueError):
        abi.selection_struct(3, np.zeros(3), np.zeros((3, 6)))
    s = abi.selection_struct(2, np.zeros(2), np.zeros((2, 7)))
    assert s.pso_cost is None and s.svi_mu is None


class _FakeCtx:
    """Records the lcf_finalize_batch inputs and answers with the oracle."""

    def __init__(self, oracle):
        self.oracle = oracle
        self.calls = []

    def finalize_batch(self, batch, model, pso, cost, per_chi2, mu, ls, elbo, method):
        self.calls.append((batch, np.array(model), np.array(pso), mu is not None))
        return self.oracle.finalize_batch(batch, model, pso, cost, per_chi2, mu, ls, elbo, method=method)


def _flux_bands(batch, s):
    out = {}
    for k, (t, f, e) in enumerate(batch.bands_of(s)):
        out["gri"[k]] = {"times": list(t), "values": list(f), "errors": list(e)}
    return out


def test_python_mirror_pairs_results_in_count_order(oracle):
    """finalize_parametric_from_gpu pairs gpu_results[i] with the i-th band in
    descending observation count, stops at the shorter list and skips an
    entry with empty pso_params (src/parametric.rs:3184-3199)."""
    from lightcurve_fitting_gb300 import parametric
    batch = synth.config_uneven(3, seed=79)
    ref = oracle.fit_batch(batch, fit_all_models=True, method=abi.METHOD_LAPLACE, run_multi_bazin=False)
    s = 0
    fb = _flux_bands(batch, s)
    b0 = batch.source_band_offsets[s]
    order = sorted(range(3), key=lambda k: -len(fb["gri"[k]]["values"]))
    gpu = []
    for k in order:
        b = b0 + k
        m = int(ref.model[b])
        gpu.append({"model": abi.MODEL_NAMES[m], "pso_params": list(ref.pso_params[b, :abi.N_PARAMS[m]]),
                    "pso_cost": float(ref.pso_chi2[b]), "per_model_chi2": {abi.MODEL_NAMES[m]: 1.0}})
    gpu[1] = dict(gpu[1], pso_params=[])
    ctx = _FakeCtx(oracle)
    rows = parametric.finalize_parametric_from_gpu(fb, gpu, method="laplace", ctx=ctx)
    assert [r["band"] for r in rows] == ["gri"[order[0]], "gri"[order[2]]]
    for r, k in zip(rows, [order[0], order[2]]):
        b = b0 + k
        n = abi.N_PARAMS[int(ref.model[b])]
        assert np.array_equal(r["svi_mu"], ref.svi_mu[b, :n])
        assert r["uncertainty_method"] == "Laplace" and r["per_model_chi2"]
    assert len(ctx.calls) == 1 and ctx.calls[0][0].n_bands == 2 and not ctx.calls[0][3]
    # two results for three bands: the third band is not finalised
    assert len(parametric.finalize_parametric_from_gpu(fb, gpu[:1], method="laplace", ctx=ctx)) == 1


def test_python_mirror_all_models_entries(oracle):
    """finalize_all_models_with_gpu_svi: one row per (gpu result, svi output,
    band name) entry; unknown band names and empty SVI outputs are skipped."""
    from lightcurve_fitting_gb300 import parametric
    batch = synth.config_basic(1, seed=83)
    fb = _flux_bands(batch, 0)
    t, f, e = batch.bands_of(0)[0]
    gpu, svi, names = [], [], []
    for m in (0, 3):
        n = abi.N_PARAMS[m]
        p = [float(x) for x in oracle.fit_batch(batch, fit_all_models=True, method=abi.METHOD_LAPLACE,
                                                 run_multi_bazin=False).per_model_params[0, m, :n]]
        u = oracle.svi_fit(m, oracle.Band(t, f, e), p)
        gpu.append({"model": abi.MODEL_NAMES[m], "pso_params": p, "pso_cost": 1.0, "per_model_chi2": {}})
        svi.append((list(u[0]), list(u[1]), u[2]))
        names.append("g")
    gpu.append(gpu[0]); svi.append(svi[0]); names.append("z")          # unknown band
    gpu.append(gpu[0]); svi.append(([], [], 0.0)); names.append("g")    # empty SVI output
    ctx = _FakeCtx(oracle)
    rows = parametric.finalize_all_models_with_gpu_svi(fb, gpu, svi, names, ctx=ctx)
    assert [r["model"] for r in rows] == ["Bazin", "Arnett"]
    assert all(r["svi_elbo"] == pytest.approx(s[2]) for r, s in zip(rows, svi))
    assert ctx.calls[0][3]


def test_bench_pair_batch_repeats_each_band_per_fitted_model(oracle):
    """The finalisation leg's input: one one-band source per fitted (band,
    model) pair, holding that band's observations and that model's polished
    parameters and cost."""
    import bench
    batch = synth.config_uneven(4, seed=101)
    res = oracle.fit_batch(batch, fit_all_models=True, method=abi.METHOD_LAPLACE, run_multi_bazin=False)
    pairs, model, pso, cost = bench.pair_batch(batch, res, 3)
    nb3 = int(batch.source_band_offsets[3])
    fitted = [(b, m) for b in range(nb3) for m in range(8)
              if res.model[b] >= 0 and np.isfinite(res.per_model_params[b, m, 0])]
    assert pairs.n_bands == pairs.n_sources == len(fitted) == model.size
    for i, (b, m) in enumerate(fitted):
        o0, o1 = batch.band_obs_offsets[b], batch.band_obs_offsets[b + 1]
        q0, q1 = pairs.band_obs_offsets[i], pairs.band_obs_offsets[i + 1]
        assert np.array_equal(pairs.times[q0:q1], batch.times[o0:o1])
        assert np.array_equal(pairs.flux[q0:q1], batch.flux[o0:o1])
        assert model[i] == m and np.array_equal(pso[i], res.per_model_params[b, m], equal_nan=True)
        assert cost[i] == res.per_model_chi2[b, m]
