"""ctypes mirrors of the structs in include/lcf.h and a host-side output
container.  Shared by the library binding (``lightcurve_fitting_gb300.lib``)
and by the test oracle's binding, so both fill identical arrays."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

N_MODELS = 8
MAX_PARAMS = 7
MB_MAX_K = 4
MB_MAX_PARAMS = 18

# status codes of include/lcf.h
LCF_OK = 0
LCF_E_INVALID = -1
LCF_E_CUDA = -2
LCF_E_NOMEM = -3
LCF_E_TIMEOUT = -4
LCF_E_UNSUPPORTED = -5
LCF_E_CAPACITY = -6
METHOD_SVI = 0
METHOD_LAPLACE = 1

# model ids, src/gpu_types.rs:51-62 and src/parametric.rs:3279-3288
MODEL_NAMES = ["Bazin", "Villar", "Tde", "Arnett", "Magnetar", "ShockCooling", "Afterglow", "MetzgerKN"]
MODEL_IDS = {n: i for i, n in enumerate(MODEL_NAMES)}
N_PARAMS = [6, 7, 7, 5, 5, 5, 6, 5]
SE_IDX = [5, 6, 6, 4, 4, 4, 5, 4]
T0_IDX = [2, 3, 2, 1, 1, 1, 1, 3]

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)


class BandsCSR(C.Structure):
    _fields_ = [
        ("n_sources", C.c_int32),
        ("n_bands", C.c_int32),
        ("source_band_offsets", C.c_void_p),
        ("band_obs_offsets", C.c_void_p),
        ("times", C.c_void_p),
        ("flux", C.c_void_p),
        ("flux_err", C.c_void_p),
    ]


class FitOptions(C.Structure):
    _fields_ = [
        ("fit_all_models", C.c_int32),
        ("method", C.c_int32),
        ("forced_model", C.c_int32),
        ("run_multi_bazin", C.c_int32),
        ("joint_multiband", C.c_int32),
    ]


class PsoSelection(C.Structure):
    """lcf_pso_selection: caller-selected fits, one row per CSR band."""
    _fields_ = [
        ("model", C.c_void_p),
        ("pso_params", C.c_void_p),
        ("pso_cost", C.c_void_p),
        ("per_model_chi2", C.c_void_p),
        ("svi_mu", C.c_void_p),
        ("svi_log_sigma", C.c_void_p),
        ("svi_elbo", C.c_void_p),
    ]


class FitOutputs(C.Structure):
    _fields_ = [
        ("model", C.c_void_p),
        ("rank", C.c_void_p),
        ("n_obs", C.c_void_p),
        ("pso_params", C.c_void_p),
        ("pso_chi2", C.c_void_p),
        ("svi_mu", C.c_void_p),
        ("svi_log_sigma", C.c_void_p),
        ("svi_elbo", C.c_void_p),
        ("mag_chi2", C.c_void_p),
        ("per_model_chi2", C.c_void_p),
        ("per_model_params", C.c_void_p),
        ("mb_best_k", C.c_void_p),
        ("mb_params", C.c_void_p),
        ("mb_cost", C.c_void_p),
        ("mb_bic", C.c_void_p),
        ("mb_per_k_cost", C.c_void_p),
        ("mb_per_k_bic", C.c_void_p),
    ]


class FitStats(C.Structure):
    _fields_ = [
        ("ms_total", C.c_double),
        ("ms_pso", C.c_double),
        ("ms_lbfgs", C.c_double),
        ("ms_t0_search", C.c_double),
        ("ms_uncertainty", C.c_double),
        ("ms_refine", C.c_double),
        ("ms_multi_bazin", C.c_double),
        ("particle_obs_evals", C.c_double),
        ("ode_steps", C.c_double),
        ("pso_tasks", C.c_int64),
        ("kernel_launches", C.c_int64),
        ("h2d_bytes", C.c_double),
        ("d2h_bytes", C.c_double),
        ("pso0_evals_by_kind", C.c_double * 12),
        ("pso0_particles_by_kind", C.c_double * 12),
        ("lbfgs_polishes", C.c_double),
        ("lbfgs_iters", C.c_double),
        ("lbfgs_evals", C.c_double),
        ("lbfgs_obs_evals", C.c_double),
        ("lbfgs_obs_evals_by_model", C.c_double * 8),
        ("ms_joint", C.c_double),
        ("lbfgs_fp64_obs_evals_by_model", C.c_double * 8),
    ]


def ptr(a: np.ndarray) -> int:
    return a.ctypes.data


@dataclass
class FitResult:
    """Per-band outputs (caller band order) of one batch fit."""

    n_bands: int
    model: np.ndarray = field(init=False)
    rank: np.ndarray = field(init=False)
    n_obs: np.ndarray = field(init=False)
    pso_params: np.ndarray = field(init=False)
    pso_chi2: np.ndarray = field(init=False)
    svi_mu: np.ndarray = field(init=False)
    svi_log_sigma: np.ndarray = field(init=False)
    svi_elbo: np.ndarray = field(init=False)
    mag_chi2: np.ndarray = field(init=False)
    per_model_chi2: np.ndarray = field(init=False)
    per_model_params: np.ndarray = field(init=False)
    mb_best_k: np.ndarray = field(init=False)
    mb_params: np.ndarray = field(init=False)
    mb_cost: np.ndarray = field(init=False)
    mb_bic: np.ndarray = field(init=False)
    mb_per_k_cost: np.ndarray = field(init=False)
    mb_per_k_bic: np.ndarray = field(init=False)

    def __post_init__(self):
        nb = self.n_bands
        nan = lambda *s: np.full(s, np.nan)
        self.model = np.full(nb, -1, np.int32)
        self.rank = np.full(nb, -1, np.int32)
        self.n_obs = np.zeros(nb, np.int32)
        self.pso_params = nan(nb, MAX_PARAMS)
        self.pso_chi2 = nan(nb)
        self.svi_mu = nan(nb, MAX_PARAMS)
        self.svi_log_sigma = nan(nb, MAX_PARAMS)
        self.svi_elbo = nan(nb)
        self.mag_chi2 = nan(nb)
        self.per_model_chi2 = nan(nb, N_MODELS)
        self.per_model_params = nan(nb, N_MODELS, MAX_PARAMS)
        self.mb_best_k = np.zeros(nb, np.int32)
        self.mb_params = nan(nb, MB_MAX_PARAMS)
        self.mb_cost = nan(nb)
        self.mb_bic = nan(nb)
        self.mb_per_k_cost = nan(nb, MB_MAX_K)
        self.mb_per_k_bic = nan(nb, MB_MAX_K)

    def as_struct(self) -> FitOutputs:
        o = FitOutputs()
        for name, _ in FitOutputs._fields_:
            setattr(o, name, ptr(getattr(self, name)))
        return o

    def bytes(self) -> int:
        return sum(getattr(self, n).nbytes for n, _ in FitOutputs._fields_)


def csr_struct(batch, keep=None) -> BandsCSR:
    """BandsCSR over the arrays of a ``PhotometryBatch`` (host pointers).
    ``keep`` collects the contiguous arrays so they outlive the struct."""
    arrs = [
        np.ascontiguousarray(batch.source_band_offsets, dtype=np.int32),
        np.ascontiguousarray(batch.band_obs_offsets, dtype=np.int64),
        np.ascontiguousarray(batch.times, dtype=np.float64),
        np.ascontiguousarray(batch.flux, dtype=np.float64),
        np.ascontiguousarray(batch.flux_err, dtype=np.float64),
    ]
    if keep is not None:
        keep.extend(arrs)
    s = BandsCSR()
    s.n_sources = batch.n_sources
    s.n_bands = batch.n_bands
    s.source_band_offsets, s.band_obs_offsets, s.times, s.flux, s.flux_err = [ptr(a) for a in arrs]
    return s


def options(fit_all_models=True, method=METHOD_SVI, forced_model=-1, run_multi_bazin=True,
            joint_multiband=False) -> FitOptions:
    o = FitOptions()
    o.fit_all_models = int(bool(fit_all_models))
    o.method = int(method)
    o.forced_model = int(forced_model)
    o.run_multi_bazin = int(bool(run_multi_bazin))
    o.joint_multiband = int(bool(joint_multiband))
    return o


def selection_struct(n_bands, model, pso_params, pso_cost=None, per_model_chi2=None, svi_mu=None,
                     svi_log_sigma=None, svi_elbo=None, keep=None) -> PsoSelection:
    """PsoSelection over host arrays: model [n_bands] (-1 skips a band),
    pso_params [n_bands, 7], optional pso_cost [n_bands], per_model_chi2
    [n_bands, 8], svi_mu / svi_log_sigma [n_bands, 7], svi_elbo [n_bands]."""
    def arr(a, dtype, shape):
        if a is None:
            return None
        v = np.ascontiguousarray(a, dtype=dtype)
        if v.size != int(np.prod(shape)):
            raise ValueError(f"selection array of size {v.size}, expected shape {shape}")
        return v
    fields = [arr(model, np.int32, (n_bands,)), arr(pso_params, np.float64, (n_bands, 7)),
              arr(pso_cost, np.float64, (n_bands,)), arr(per_model_chi2, np.float64, (n_bands, 8)),
              arr(svi_mu, np.float64, (n_bands, 7)), arr(svi_log_sigma, np.float64, (n_bands, 7)),
              arr(svi_elbo, np.float64, (n_bands,))]
    if keep is not None:
        keep.extend(f for f in fields if f is not None)
    s = PsoSelection()
    (s.model, s.pso_params, s.pso_cost, s.per_model_chi2, s.svi_mu, s.svi_log_sigma,
     s.svi_elbo) = [ptr(f) if f is not None else None for f in fields]
    return s
