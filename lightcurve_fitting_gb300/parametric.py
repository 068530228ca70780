"""Python mirror of the reference's parametric API on the GB300 kernels.

Names, arguments and return values follow the reference's Python binding
(python/src/lib.rs:203-245) and its Rust API (src/parametric.rs:3563-3761):
results are lists of dicts with the fields of ``ParametricBandResult``
(src/parametric.rs:3049-3072), ``None`` where the reference has ``None``.

Every call runs on the GPU through liblcf_gb300.so; there is no CPU path.
``fit_parametric`` with ``fit_all_models=False`` dispatches a source with
two or more non-empty bands to the joint multi-band Villar fit
(src/parametric.rs:3750-3757, fit_parametric_multiband :3815-4131), as the
reference does.
"""
from __future__ import annotations

import math
from typing import Dict, List, Sequence

import numpy as np

from . import abi
from .lib import default_context
from .synth import PhotometryBatch

FACTOR = 1.0857362047581294


def _method(method: str) -> int:
    m = method.lower() if isinstance(method, str) else method
    if m == "svi":
        return abi.METHOD_SVI
    if m == "laplace":
        return abi.METHOD_LAPLACE
    raise ValueError(f"Unknown uncertainty method '{method}'. Expected 'svi' or 'laplace'.")


def _model_id(name: str) -> int:
    table = {"bazin": 0, "villar": 1, "tde": 2, "arnett": 3, "magnetar": 4, "shockcooling": 5,
             "afterglow": 6, "metzgerkn": 7}
    key = name.lower()
    if key not in table:
        raise ValueError(f"Unknown model '{name}'. Expected one of: Bazin, Villar, Tde, Arnett, Magnetar, "
                         "ShockCooling, Afterglow, MetzgerKN.")
    return table[key]


def build_flux_bands(times, mags, mag_errs, bands) -> Dict[str, dict]:
    """build_flux_bands (src/common.rs:79-111): group by band, times relative to
    the earliest time, mag -> flux with ZP 23.9, drop non-finite or <= 0."""
    times = np.asarray(times, np.float64)
    if times.size == 0:
        return {}
    jd_min = times.min()
    out: Dict[str, dict] = {}
    for t, m, e, b in zip(times, mags, mag_errs, bands):
        flux = 10.0 ** (-0.4 * (m - 23.9))
        ferr = e / FACTOR * flux
        if not (math.isfinite(flux) and math.isfinite(ferr)) or flux <= 0 or ferr <= 0:
            continue
        d = out.setdefault(b, {"times": [], "values": [], "errors": []})
        d["times"].append(t - jd_min)
        d["values"].append(flux)
        d["errors"].append(ferr)
    return out


def build_raw_flux_bands(times, fluxes, flux_errs, bands) -> Dict[str, dict]:
    """build_raw_flux_bands (src/common.rs:117-149): linear fluxes grouped by
    band, times relative to the earliest time, non-finite or <= 0 values and
    errors dropped."""
    times = np.asarray(times, np.float64)
    if times.size == 0:
        return {}
    jd_min = times.min()
    out: Dict[str, dict] = {}
    for t, f, e, b in zip(times, fluxes, flux_errs, bands):
        f, e = float(f), float(e)
        if not (math.isfinite(f) and math.isfinite(e)) or f <= 0 or e <= 0:
            continue
        d = out.setdefault(b, {"times": [], "values": [], "errors": []})
        d["times"].append(float(t) - jd_min)
        d["values"].append(f)
        d["errors"].append(e)
    return out


def _batch_from_sources(sources: Sequence[Dict[str, dict]]):
    t, f, e, bo, so, names = [], [], [], [0], [0], []
    for bands in sources:
        keys = list(bands.keys())
        names.append(keys)
        for k in keys:
            bd = bands[k]
            tt = np.asarray(bd["times"], np.float64)
            t.append(tt)
            f.append(np.asarray(bd["values"], np.float64))
            e.append(np.asarray(bd["errors"], np.float64))
            bo.append(bo[-1] + tt.size)
        so.append(so[-1] + len(keys))
    cat = lambda xs: np.concatenate(xs) if xs else np.zeros(0)
    batch = PhotometryBatch(cat(t), cat(f), cat(e), np.asarray(bo, np.int64), np.asarray(so, np.int32),
                            np.zeros(len(sources), np.int32), "api")
    return batch, names


def _opt(v: float):
    return None if v is None or not math.isfinite(v) else float(v)


def results_from_fit(res: abi.FitResult, batch: PhotometryBatch, names, fit_all_models: bool, method: int,
                     forced_model: int, joint=None) -> List[List[dict]]:
    """Per source: the list of ParametricBandResult dicts in the reference's
    band order (descending observation count); joint[s] marks the sources of
    the joint multi-band fit."""
    joint = joint if joint is not None else [False] * batch.n_sources
    out = []
    for s in range(batch.n_sources):
        b0, b1 = int(batch.source_band_offsets[s]), int(batch.source_band_offsets[s + 1])
        rows = []
        for b in range(b0, b1):
            if res.model[b] < 0:
                continue
            m = int(res.model[b])
            np_ = abi.N_PARAMS[m]
            if forced_model >= 0:
                chi2 = {abi.MODEL_NAMES[forced_model]: _opt(res.per_model_chi2[b, forced_model])}
            elif joint[s]:
                chi2 = {abi.MODEL_NAMES[1]: _opt(res.per_model_chi2[b, 1])}  # the joint fit: Villar only
            else:
                chi2 = {abi.MODEL_NAMES[k]: _opt(res.per_model_chi2[b, k]) for k in range(8)}
            per_params = {}
            if fit_all_models:
                for k in range(8):
                    row = res.per_model_params[b, k, :abi.N_PARAMS[k]]
                    if not np.all(np.isnan(row)):
                        per_params[abi.MODEL_NAMES[k]] = [float(x) for x in row]
            r = {
                "band": names[s][b - b0],
                "model": abi.MODEL_NAMES[m],
                "pso_params": [float(x) for x in res.pso_params[b, :np_]],
                "pso_chi2": _opt(res.pso_chi2[b]),
                "svi_mu": [float(x) for x in res.svi_mu[b, :np_]],
                "svi_log_sigma": [float(x) for x in res.svi_log_sigma[b, :np_]],
                "svi_elbo": _opt(res.svi_elbo[b]),
                "n_obs": int(res.n_obs[b]),
                "mag_chi2": _opt(res.mag_chi2[b]),
                "per_model_chi2": chi2,
                "uncertainty_method": "Svi" if method == abi.METHOD_SVI else "Laplace",
            }
            if per_params:
                r["per_model_params"] = per_params
            if res.mb_best_k[b] > 0:
                k = int(res.mb_best_k[b])
                r["multi_bazin"] = {
                    "best_k": k,
                    "params": [float(x) for x in res.mb_params[b, :4 * k + 2]],
                    "cost": float(res.mb_cost[b]),
                    "bic": float(res.mb_bic[b]),
                    "per_k_cost": [float(x) for x in res.mb_per_k_cost[b]],
                    "per_k_bic": [float(x) for x in res.mb_per_k_bic[b]],
                }
            rows.append((int(res.rank[b]), r))
        rows.sort(key=lambda x: x[0])
        out.append([r for _, r in rows])
    return out


def fit_batch_parametric(sources: Sequence[Dict[str, dict]], fit_all_models: bool = False, method: str = "svi",
                         model: str | None = None, ctx=None) -> List[List[dict]]:
    """fit_batch_parametric (src/batch.rs:39-48) of the per-band model
    selection path: one list of band results per source, all sources in one
    GPU batch."""
    meth = _method(method)
    forced = -1 if model is None else _model_id(model)
    joint_on = forced < 0 and not fit_all_models
    joint = [joint_on and sum(1 for b in bands.values() if len(b["values"]) > 0) >= 2 for bands in sources]
    batch, names = _batch_from_sources(sources)
    ctx = ctx or default_context()
    res = ctx.fit_batch(batch, fit_all_models=fit_all_models, method=meth, forced_model=forced,
                        run_multi_bazin=True, joint_multiband=joint_on)
    return results_from_fit(res, batch, names, fit_all_models, meth, forced, joint)


def fit_parametric(bands: Dict[str, dict], fit_all_models: bool = False, method: str = "svi", ctx=None):
    """fit_parametric (src/parametric.rs:3742-3761, python/src/lib.rs:203-215)."""
    return fit_batch_parametric([bands], fit_all_models, method, None, ctx)[0]


def fit_parametric_model(bands: Dict[str, dict], model: str, fit_all_models: bool = False, method: str = "svi",
                         ctx=None):
    """fit_parametric_model with a forced model (python/src/lib.rs:219-245)."""
    return fit_batch_parametric([bands], fit_all_models, method, model, ctx)[0]


# ---------------------------------------------------------------------------
# Batched finalisation of externally selected fits (lcf_finalize_batch):
# finalize_parametric_from_gpu, finalize_parametric_with_gpu_svi and
# finalize_all_models_with_gpu_svi (src/parametric.rs:3126-3553).  A
# ``gpu_results`` entry is a dict with the fields of GpuPsoBandResult
# (:3101-3114): "model" (name), "pso_params", "pso_cost", "per_model_chi2"
# (name -> value or None), optionally "per_model_params" and "multi_bazin".
# An ``svi_outputs`` entry is (mu, log_sigma, elbo).
# ---------------------------------------------------------------------------
def _fittable(bd: dict) -> bool:
    v = np.asarray(bd["values"], np.float64)
    return v.size > 0 and float(np.max(v)) > 0.0


def _finalize_run(entries, gpu_rows, svi_rows, method: int, ctx):
    """One lcf_finalize_batch call over (band dict, gpu result, svi output or
    None) triples, each its own source; returns the FitResult."""
    t, f, e, bo = [], [], [], [0]
    nb = len(entries)
    model = np.full(nb, -1, np.int32)
    pso = np.full((nb, 7), np.nan)
    cost = np.full(nb, np.nan)
    given = svi_rows is not None
    mu = np.full((nb, 7), np.nan) if given else None
    ls = np.full((nb, 7), np.nan) if given else None
    elbo = np.full(nb, np.nan) if given else None
    for i, bd in enumerate(entries):
        tt = np.asarray(bd["times"], np.float64)
        t.append(tt)
        f.append(np.asarray(bd["values"], np.float64))
        e.append(np.asarray(bd["errors"], np.float64))
        bo.append(bo[-1] + tt.size)
        g = gpu_rows[i]
        m = _model_id(g["model"])
        n = abi.N_PARAMS[m]
        p = np.asarray(g["pso_params"], np.float64)
        model[i] = m
        pso[i, :min(n, p.size)] = p[:n]
        pc = g.get("pso_cost")
        cost[i] = np.nan if pc is None else float(pc)
        if given:
            smu, sls, sel = svi_rows[i]
            mu[i, :n] = np.asarray(smu, np.float64)[:n]
            ls[i, :n] = np.asarray(sls, np.float64)[:n]
            elbo[i] = sel
    cat = lambda xs: np.concatenate(xs) if xs else np.zeros(0)
    batch = PhotometryBatch(cat(t), cat(f), cat(e), np.asarray(bo, np.int64), np.arange(nb + 1, dtype=np.int32),
                            np.zeros(nb, np.int32), "finalize")
    ctx = ctx or default_context()
    return ctx.finalize_batch(batch, model, pso, cost, None, mu, ls, elbo, method=method)


def _finalized(res, i, name, g, method: int, per_params, mb):
    m = int(res.model[i])
    n = abi.N_PARAMS[m]
    r = {
        "band": name,
        "model": abi.MODEL_NAMES[m],
        "pso_params": [float(x) for x in np.asarray(g["pso_params"], np.float64)],
        "pso_chi2": _opt(g.get("pso_cost")),
        "svi_mu": [float(x) for x in res.svi_mu[i, :n]],
        "svi_log_sigma": [float(x) for x in res.svi_log_sigma[i, :n]],
        "svi_elbo": _opt(res.svi_elbo[i]),
        "n_obs": int(res.n_obs[i]),
        "mag_chi2": _opt(res.mag_chi2[i]),
        "per_model_chi2": dict(g.get("per_model_chi2") or {}),
        "uncertainty_method": "Svi" if method == abi.METHOD_SVI else "Laplace",
    }
    if per_params:
        r["per_model_params"] = per_params
    if mb is not None:
        r["multi_bazin"] = mb
    return r


def _sorted_entries(flux_bands: Dict[str, dict]):
    """fit_parametric_model's band preparation order: fittable bands by
    observation count, descending (ties in the dict's order)."""
    names = [k for k, bd in flux_bands.items() if _fittable(bd)]
    return sorted(names, key=lambda k: -len(flux_bands[k]["values"]))


def _finalize_sorted(flux_bands, gpu_results, svi_outputs, method: int, ctx):
    names = _sorted_entries(flux_bands)
    pairs = []
    for idx, name in enumerate(names):
        if idx >= len(gpu_results) or (svi_outputs is not None and idx >= len(svi_outputs)):
            break
        if len(gpu_results[idx]["pso_params"]) == 0:
            continue
        pairs.append((idx, name))
    if not pairs:
        return []
    res = _finalize_run([flux_bands[n] for _, n in pairs], [gpu_results[i] for i, _ in pairs],
                        None if svi_outputs is None else [svi_outputs[i] for i, _ in pairs], method, ctx)
    out = []
    for k, (idx, name) in enumerate(pairs):
        g = gpu_results[idx]
        out.append(_finalized(res, k, name, g, method, g.get("per_model_params") or {},
                              g.get("multi_bazin") if idx == 0 else None))
    return out


def finalize_parametric_from_gpu(flux_bands: Dict[str, dict], gpu_results: Sequence[dict], method: str = "svi",
                                 ctx=None) -> List[dict]:
    """finalize_parametric_from_gpu (src/parametric.rs:3126-3257): per band,
    in the by-count order, SVI from (or Laplace at) the supplied PSO
    parameters, then the refinements and the magnitude chi2."""
    if not flux_bands or not gpu_results:
        return []
    return _finalize_sorted(flux_bands, gpu_results, None, _method(method), ctx)


def finalize_parametric_with_gpu_svi(flux_bands: Dict[str, dict], gpu_results: Sequence[dict],
                                     svi_outputs: Sequence[tuple], ctx=None) -> List[dict]:
    """finalize_parametric_with_gpu_svi (src/parametric.rs:3298-3421): the
    same from supplied SVI outputs."""
    if not flux_bands or not gpu_results or not svi_outputs:
        return []
    return _finalize_sorted(flux_bands, gpu_results, svi_outputs, abi.METHOD_SVI, ctx)


def finalize_all_models_with_gpu_svi(flux_bands: Dict[str, dict], gpu_results: Sequence[dict],
                                     svi_outputs: Sequence[tuple], band_names: Sequence[str], ctx=None) -> List[dict]:
    """finalize_all_models_with_gpu_svi (src/parametric.rs:3429-3553): one
    result per (band, model) entry; band_names[i] names entry i's band."""
    if not flux_bands or not gpu_results or not svi_outputs:
        return []
    picks = []
    for idx, g in enumerate(gpu_results):
        if idx >= len(svi_outputs) or idx >= len(band_names):
            break
        name = band_names[idx]
        if name not in flux_bands or not _fittable(flux_bands[name]):
            continue
        if len(g["pso_params"]) == 0 or len(svi_outputs[idx][0]) == 0:
            continue
        picks.append(idx)
    if not picks:
        return []
    res = _finalize_run([flux_bands[band_names[i]] for i in picks], [gpu_results[i] for i in picks],
                        [svi_outputs[i] for i in picks], abi.METHOD_SVI, ctx)
    return [_finalized(res, k, band_names[i], gpu_results[i], abi.METHOD_SVI, {}, gpu_results[i].get("multi_bazin"))
            for k, i in enumerate(picks)]


def fit_parametric_multiband(bands: Dict[str, dict], method: str = "svi", ctx=None) -> List[dict]:
    """fit_parametric_multiband (python/src/lib.rs:257-269, src/parametric.rs:3813-4131):
    the joint multi-band Villar fit of one source, then per-band uncertainty,
    refinements and MultiBazin.  The library's joint swarm fits 2 to 6
    non-empty bands; a source with fewer raises ValueError (the reference
    runs its joint swarm on a single band too)."""
    meth = _method(method)
    if not bands:
        return []
    if sum(1 for b in bands.values() if len(b["values"]) > 0) < 2:
        raise ValueError("fit_parametric_multiband needs at least two non-empty bands")
    batch, names = _batch_from_sources([bands])
    ctx = ctx or default_context()
    res = ctx.fit_batch(batch, fit_all_models=False, method=meth, forced_model=-1, run_multi_bazin=True,
                        joint_multiband=True)
    return results_from_fit(res, batch, names, False, meth, -1, [True])[0]


_EVAL_EXPORTS = ["launch_bazin", "launch_villar", "launch_tde", "launch_arnett", "launch_magnetar",
                 "launch_shock_cooling", "launch_afterglow", "launch_metzger_kn"]


def eval_model(model: str, params, times) -> List[float]:
    """eval_model (python/src/lib.rs:316-326, eval_model_flux
    src/parametric.rs:3082-3097): the model's normalised flux at `times`
    from the internal parameter vector, evaluated on the GPU by the
    library's drop-in launch_* kernels (MetzgerKN: one ODE over all times)."""
    import torch
    from .lib import load
    m = _model_id(model)
    p = np.asarray(params, np.float64)
    t = np.asarray(times, np.float64)
    if p.size < abi.N_PARAMS[m]:
        raise ValueError(f"{abi.MODEL_NAMES[m]} takes {abi.N_PARAMS[m]} parameters, got {p.size}")
    if t.size == 0:
        return []
    L = load()
    dev = torch.device("cuda", torch.cuda.current_device())
    dp = torch.from_numpy(p).to(dev)
    dt = torch.from_numpy(t).to(dev)
    do = torch.empty(t.size, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    getattr(L, _EVAL_EXPORTS[m])(dp.data_ptr(), dt.data_ptr(), do.data_ptr(), 1, int(t.size), int(p.size), 1, 256)
    torch.cuda.synchronize()
    return [float(x) for x in do.cpu().numpy()]
