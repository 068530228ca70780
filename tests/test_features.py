"""Parametric features (src/features.rs:264-362) from fit results: the oracle
fits a few sources, parametric.results_from_fit turns them into the
reference's ParametricBandResult dicts, and the features are checked against
the definitions."""
import math

import numpy as np

from lightcurve_fitting_gb300 import abi, features, parametric, synth


def _results(oracle, fit_all_models=True, joint=False):
    b = synth.config_basic(3, seed=7)
    names = [["g", "r", "i"] for _ in range(b.n_sources)]
    res = oracle.fit_batch(b, fit_all_models=fit_all_models, method=abi.METHOD_LAPLACE, joint_multiband=joint)
    return parametric.results_from_fit(res, b, names, fit_all_models, abi.METHOD_LAPLACE, -1,
                                       [joint] * b.n_sources)


def test_param_features_follow_the_definitions(oracle):
    for src in _results(oracle):
        f = features.extract_param_features(src, "r")
        ref = next(r for r in src if r["band"] == "r")
        assert f["param_best_model"] == features.MODEL_INT[ref["model"]]
        assert f["param_n_obs"] == ref["n_obs"] and f["param_n_bands_fit"] == len(src)
        assert f["param_svi_mu_0"] == ref["svi_mu"][0]
        assert math.isclose(f["param_svi_sigma_mean"], np.mean(np.exp(ref["svi_log_sigma"])))
        chi2 = sorted(r["pso_chi2"] for r in src)
        assert math.isclose(f["param_delta_chi2"], chi2[1] - chi2[0])
        for name in features.ALL_MODELS:
            mc = ref["per_model_chi2"][name]
            assert f[f"param_chi2_{name}"] == mc
            if mc is not None:
                assert math.isclose(f[f"param_dchi2_{name}"], mc - ref["pso_chi2"], abs_tol=1e-15)
        if ref["model"] == "Bazin":
            assert math.isclose(f["param_bazin_rise_tau"], math.exp(ref["pso_params"][3]))
        else:
            assert f["param_bazin_rise_tau"] is None
        mb = ref.get("multi_bazin")
        assert (f["mb_best_k"] is None) == (mb is None)
        assert len(f) == 34  # the reference's 34 parametric and MultiBazin keys


def test_param_features_fall_back_to_the_first_band_and_handle_empty(oracle):
    src = _results(oracle)[0]
    f = features.extract_param_features(src, "z")  # no such band: the first result
    assert f["param_n_obs"] == src[0]["n_obs"]
    assert features.extract_param_features([], "r") == {}


def test_param_features_of_the_joint_fit(oracle):
    src = _results(oracle, fit_all_models=False, joint=True)[0]
    f = features.extract_param_features(src, "r")
    assert f["param_best_model"] == 1.0 and f["param_delta_chi2"] == 0.0  # one joint cost for all bands
    assert f["param_chi2_Villar"] == f["param_pso_chi2"] and f["param_dchi2_Villar"] == 0.0
    assert all(f[f"param_chi2_{m}"] is None for m in features.ALL_MODELS if m != "Villar")
