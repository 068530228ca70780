"""Parametric features of a source from its fit results, as the reference's
extract_param_features / extract_mb_features (src/features.rs:264-362, model
codes and names :26-61): the downstream consumer of fit_parametric in the
reference's feature pipeline (extract_features_from_results, :477-492).

The input is the list of ParametricBandResult dicts that
``parametric.fit_parametric`` / ``fit_batch_parametric`` return; the output is
the reference's FeatureMap as a dict (``None`` where the reference has
``None``).  Host-side only: the features are a few arithmetic operations per
source.
"""
from __future__ import annotations

import math
from typing import Dict, List, Optional, Sequence

# model codes and the order of the per-model features, src/features.rs:26-61
MODEL_INT = {"Bazin": 0, "Villar": 1, "MetzgerKN": 2, "Tde": 3, "Arnett": 4, "Magnetar": 5, "ShockCooling": 6,
             "Afterglow": 7}
ALL_MODELS = ["Bazin", "Villar", "MetzgerKN", "Tde", "Arnett", "Magnetar", "ShockCooling", "Afterglow"]


def _opt(v) -> Optional[float]:
    return float(v) if v is not None and math.isfinite(v) else None


def _mb_features(mb: Optional[dict], f: Dict[str, Optional[float]]) -> None:
    """extract_mb_features, src/features.rs:341-362."""
    if mb is None:
        for k in ("mb_best_k", "mb_cost", "mb_bic", "mb_bic_improvement_k2"):
            f[k] = None
        return
    f["mb_best_k"] = float(mb["best_k"])
    f["mb_cost"] = _opt(mb["cost"])
    f["mb_bic"] = _opt(mb["bic"])
    pkb = mb.get("per_k_bic", [])
    ok = len(pkb) >= 2 and math.isfinite(pkb[0]) and math.isfinite(pkb[1])
    f["mb_bic_improvement_k2"] = pkb[0] - pkb[1] if ok else None


def extract_param_features(param_results: Sequence[dict], ref_band: str = "r") -> Dict[str, Optional[float]]:
    """extract_param_features, src/features.rs:264-339: features of the
    reference band's result (the first result when no band is `ref_band`);
    an empty dict when there is no result."""
    f: Dict[str, Optional[float]] = {}
    ref = next((r for r in param_results if r["band"] == ref_band), None)
    if ref is None:
        ref = param_results[0] if param_results else None
    if ref is None:
        return f
    f["param_best_model"] = float(MODEL_INT[ref["model"]])
    f["param_pso_chi2"] = _opt(ref["pso_chi2"])
    f["param_svi_elbo"] = _opt(ref["svi_elbo"])
    f["param_mag_chi2"] = _opt(ref["mag_chi2"])
    f["param_n_obs"] = float(ref["n_obs"])
    mu = ref["svi_mu"]
    for i in range(4):
        f[f"param_svi_mu_{i}"] = _opt(mu[i]) if i < len(mu) else None
    ls = ref["svi_log_sigma"]
    f["param_svi_sigma_mean"] = sum(math.exp(v) for v in ls) / len(ls) if ls else None
    if ref["model"] == "Bazin" and len(ref["pso_params"]) >= 5:
        f["param_bazin_rise_tau"] = math.exp(ref["pso_params"][3])
        f["param_bazin_decay_tau"] = math.exp(ref["pso_params"][4])
    else:
        f["param_bazin_rise_tau"] = None
        f["param_bazin_decay_tau"] = None
    chi2s = sorted(r["pso_chi2"] for r in param_results if r["pso_chi2"] is not None and math.isfinite(r["pso_chi2"]))
    f["param_delta_chi2"] = chi2s[1] - chi2s[0] if len(chi2s) >= 2 else None
    best = ref["pso_chi2"]
    for name in ALL_MODELS:
        mc = ref["per_model_chi2"].get(name)
        f[f"param_chi2_{name}"] = _opt(mc)
        both = mc is not None and best is not None and math.isfinite(mc) and math.isfinite(best)
        f[f"param_dchi2_{name}"] = mc - best if both else None
    f["param_n_bands_fit"] = float(len(param_results))
    _mb_features(ref.get("multi_bazin"), f)
    return f


def extract_param_features_batch(results: Sequence[Sequence[dict]], ref_band: str = "r") -> List[dict]:
    """extract_param_features for every source of a batch fit."""
    return [extract_param_features(r, ref_band) for r in results]
