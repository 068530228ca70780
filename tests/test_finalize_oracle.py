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
