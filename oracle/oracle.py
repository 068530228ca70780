"""TEST INFRASTRUCTURE ONLY — ctypes binding of the FP64 C++ oracle
(oracle/lcf_oracle.cpp), a restatement of the reference's CPU fitting path
(src/parametric.rs).  Only tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline / reference arm may import this module; the shipped library never
does.  The shared library is built by ``build()`` (plain g++ through
oracle/Makefile) into oracle/_build/."""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from lightcurve_fitting_gb300 import abi  # noqa: E402

LIB_PATH = os.path.join(HERE, "_build", "liblcf_oracle.so")
REF_LIB_PATH = os.path.join(HERE, "_ref", "libref_models.so")

_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle (and the reference pin harness when the reference
    checkout is present).  Returns the oracle library path."""
    # the pin harness is built only where the reference checkout exists
    # (oracle/Makefile knows where; LCF_REFERENCE_DIR overrides)
    target = ["all", "ref-if-present"]
    if force:
        subprocess.check_call(["make", "-C", HERE, "clean"], stdout=subprocess.DEVNULL)
    subprocess.check_call(["make", "-C", HERE, *target], stdout=subprocess.DEVNULL)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        d, i, u64 = C.c_double, C.c_int, C.c_uint64
        vp = C.c_void_p
        L.orc_rng_stream.argtypes = [u64, i, vp]
        L.orc_rng_f64.argtypes = [u64, i, vp]
        L.orc_log_normal_cdf.argtypes = [d]
        L.orc_log_normal_cdf.restype = d
        L.orc_erf_approx.argtypes = [d]
        L.orc_erf_approx.restype = d
        L.orc_eval_model.argtypes = [i, vp, vp, i, vp]
        L.orc_eval_grad.argtypes = [i, vp, vp, i, vp]
        L.orc_band_cost.argtypes = [i, vp, vp, vp, vp, vp, i, vp, i, i, vp]
        L.orc_band_cost_grad.argtypes = [i, vp, vp, vp, vp, vp, i, vp, vp]
        L.orc_pso_run.argtypes = [i, vp, vp, vp, vp, vp, i, vp, vp, u64, vp, i, vp]
        L.orc_pso_run.restype = d
        L.orc_lbfgs_refine.argtypes = [i, vp, vp, vp, vp, vp, i, vp, vp, vp, d]
        L.orc_lbfgs_refine.restype = d
        L.orc_svi_fit.argtypes = [i, vp, vp, vp, vp, vp, i, vp, i, i, d, vp, vp, vp]
        L.orc_laplace_fit.argtypes = [i, vp, vp, vp, vp, vp, i, vp, vp, vp]
        L.orc_model_restart.argtypes = [i, vp, vp, vp, vp, vp, i, i, vp]
        L.orc_svi_elbo_grad.argtypes = [i, vp, vp, vp, vp, vp, i, vp, vp, vp, i, vp, vp]
        L.orc_fit_batch.argtypes = [C.POINTER(abi.BandsCSR), C.POINTER(abi.FitOptions), C.POINTER(abi.FitOutputs), i]
        L.orc_finalize_batch.argtypes = [C.POINTER(abi.BandsCSR), vp, vp, vp, vp, vp, vp, vp, i,
                                         C.POINTER(abi.FitOutputs), i]
        L.orc_laplace_refine.argtypes = [i, vp, vp, vp, i, vp, vp, vp, vp]
        L.orc_svi_refine.argtypes = [i, vp, vp, vp, i, vp, vp, vp, vp]
        L.orc_joint_cost.argtypes = [C.POINTER(abi.BandsCSR), i, vp, vp]
        L.orc_pso_stats.argtypes = [vp, i]
        L.orc_max_threads.restype = i
        L.orc_set_cost_perturbation.argtypes = [d, u64, d]
        L.orc_set_position_perturbation.argtypes = [d, u64]
        L.orc_set_laplace_step.argtypes = [d]
        L.orc_metzger_at_obs.argtypes = [vp, d]
        L.orc_metzger_at_obs.restype = d
        L.orc_gpu_pso_cost.argtypes = [i, vp, vp, vp, vp, vp, i, vp, i, i, vp]
        L.orc_gpu_mb_cost.argtypes = [vp, vp, vp, vp, vp, i, vp, i, i, i, vp]
        L.orc_gpu_svi_fit.argtypes = [i, vp, vp, vp, vp, vp, i, vp, i, i, vp, vp, i, i, d, i, vp, vp, vp]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data


def rng_stream(seed: int, n: int) -> np.ndarray:
    out = np.zeros(n, np.uint64)
    lib().orc_rng_stream(seed, n, _p(out))
    return out


def rng_f64(seed: int, n: int) -> np.ndarray:
    out = np.zeros(n, np.float64)
    lib().orc_rng_f64(seed, n, _p(out))
    return out


def eval_model(model: int, params, times) -> np.ndarray:
    p = np.ascontiguousarray(params, np.float64)
    t = np.ascontiguousarray(times, np.float64)
    out = np.zeros(t.size)
    assert lib().orc_eval_model(model, _p(p), _p(t), t.size, _p(out)) == 0
    return out


def eval_grad(model: int, params, times) -> np.ndarray:
    p = np.ascontiguousarray(params, np.float64)
    t = np.ascontiguousarray(times, np.float64)
    npar = abi.N_PARAMS[model]
    out = np.zeros((t.size, npar))
    assert lib().orc_eval_grad(model, _p(p), _p(t), t.size, _p(out)) == 0
    return out


class Band:
    """A peak-normalised band (BandFitData, src/parametric.rs:3014-3025)."""

    def __init__(self, times, flux, flux_err):
        times = np.asarray(times, np.float64)
        flux = np.asarray(flux, np.float64)
        err = np.asarray(flux_err, np.float64)
        peak = np.max(flux)
        self.peak = peak
        self.t = np.ascontiguousarray(times)
        self.f = np.ascontiguousarray(flux / peak)
        self.fe = err / peak
        self.var = np.ascontiguousarray(self.fe ** 2 + 1e-10)
        self.up = np.ascontiguousarray(((err > 0) & (flux / err < 3.0)).astype(np.uint8))
        self.uf = np.ascontiguousarray(3.0 * err / peak)

    @property
    def n(self):
        return self.t.size

    def args(self):
        return (_p(self.t), _p(self.f), _p(self.var), _p(self.up), _p(self.uf), self.n)


def band_cost(model: int, band: Band, params, with_prior: bool = True) -> np.ndarray:
    p = np.ascontiguousarray(np.atleast_2d(params), np.float64)
    out = np.zeros(p.shape[0])
    assert lib().orc_band_cost(model, *band.args(), _p(p), p.shape[0], int(with_prior), _p(out)) == 0
    return out


def band_cost_grad(model: int, band: Band, params) -> np.ndarray:
    p = np.ascontiguousarray(params, np.float64)
    g = np.zeros(abi.N_PARAMS[model])
    assert lib().orc_band_cost_grad(model, *band.args(), _p(p), _p(g)) == 0
    return g


def pso_run(model: int, band: Band, lo, hi, seed: int, seed_particle=None, with_prior=True):
    lo = np.ascontiguousarray(lo, np.float64)
    hi = np.ascontiguousarray(hi, np.float64)
    g = np.zeros(abi.N_PARAMS[model])
    sp = None if seed_particle is None else np.ascontiguousarray(seed_particle, np.float64)
    c = lib().orc_pso_run(model, *band.args(), _p(lo), _p(hi), seed, None if sp is None else _p(sp),
                          int(with_prior), _p(g))
    return g, c


def model_restart(model: int, band: Band, restart: int):
    """Restart `restart` of the model-selection swarm (pso_fit_single_model):
    (cost, iterations, evaluations, best position)."""
    out = np.zeros(10)
    assert lib().orc_model_restart(model, *band.args(), int(restart), _p(out)) == 0
    return float(out[0]), int(out[1]), int(out[2]), out[3:3 + abi.N_PARAMS[model]].copy()


def svi_fit(model: int, band: Band, init, n_steps=1000, n_samples=4, lr=0.01):
    ini = np.ascontiguousarray(init, np.float64)
    npar = abi.N_PARAMS[model]
    mu, ls, elbo = np.zeros(npar), np.zeros(npar), np.zeros(1)
    steps = lib().orc_svi_fit(model, *band.args(), _p(ini), n_steps, n_samples, lr, _p(mu), _p(ls), _p(elbo))
    return mu, ls, float(elbo[0]), steps


def svi_elbo_grad(model: int, band: Band, init, vparams, eps):
    """One SVI step's ELBO estimate and its gradient (d/d mu, d/d log sigma)
    at vparams = [mu, log sigma] with the standard-normal draws eps
    [n_samples, n_params]; the prior is centred on init.  Returns
    (elbo, grad, flags): flags bit 0 = an upper-limit CDF hit its floor,
    bit 1 = a MetzgerKN sample was skipped."""
    npar = abi.N_PARAMS[model]
    ini = np.ascontiguousarray(init, np.float64)
    v = np.ascontiguousarray(vparams, np.float64)
    e = np.ascontiguousarray(eps, np.float64).reshape(-1, npar)
    assert ini.size == npar and v.size == 2 * npar
    elbo, grad = np.zeros(1), np.zeros(2 * npar)
    flags = lib().orc_svi_elbo_grad(model, *band.args(), _p(ini), _p(v), _p(e), e.shape[0], _p(elbo), _p(grad))
    assert flags >= 0
    return float(elbo[0]), grad, int(flags)


def laplace_refine(model: int, times, flux, flux_err, params):
    """Laplace at ``params``, then the profile refinements and the magnitude
    chi2 (src/parametric.rs:2464-3008, 3680-3711) on a raw band: returns
    (mu, log_sigma, mag_chi2), or None for a band the reference skips."""
    t = np.ascontiguousarray(times, np.float64)
    f = np.ascontiguousarray(flux, np.float64)
    e = np.ascontiguousarray(flux_err, np.float64)
    k = abi.N_PARAMS[model]
    p = np.ascontiguousarray(params[:k], np.float64)
    mu, ls, mag = np.zeros(k), np.zeros(k), np.zeros(1)
    rc = lib().orc_laplace_refine(int(model), _p(t), _p(f), _p(e), t.size, _p(p), _p(mu), _p(ls), _p(mag))
    return None if rc != 0 else (mu, ls, float(mag[0]))


def svi_refine(model: int, times, flux, flux_err, init):
    """SVI from ``init`` (the post-t0-search PSO parameters), then the profile
    refinements and the magnitude chi2, on a raw band: (mu, log_sigma,
    mag_chi2), or None for a band the reference skips."""
    t = np.ascontiguousarray(times, np.float64)
    f = np.ascontiguousarray(flux, np.float64)
    e = np.ascontiguousarray(flux_err, np.float64)
    k = abi.N_PARAMS[model]
    p = np.ascontiguousarray(init[:k], np.float64)
    mu, ls, mag = np.zeros(k), np.zeros(k), np.zeros(1)
    rc = lib().orc_svi_refine(int(model), _p(t), _p(f), _p(e), t.size, _p(p), _p(mu), _p(ls), _p(mag))
    return None if rc != 0 else (mu, ls, float(mag[0]))


def joint_cost(batch, src: int, p) -> float:
    """The joint multi-band cost (src/parametric.rs:3900-4001) of source
    `src` at the joint vector p (rank-0 band's Villar parameters, then the
    offsets of ranks 1, 2, ...)."""
    keep = []
    csr = abi.csr_struct(batch, keep)
    pv = np.ascontiguousarray(p, np.float64)
    out = np.zeros(1)
    nb = lib().orc_joint_cost(C.byref(csr), int(src), _p(pv), _p(out))
    return float(out[0]) if nb > 0 else float("nan")


def fit_batch(batch, fit_all_models=True, method=abi.METHOD_SVI, forced_model=-1, run_multi_bazin=True,
              n_threads=0, joint_multiband=False) -> abi.FitResult:
    keep = []
    csr = abi.csr_struct(batch, keep)
    opts = abi.options(fit_all_models, method, forced_model, run_multi_bazin, joint_multiband)
    res = abi.FitResult(batch.n_bands)
    outs = res.as_struct()
    rc = lib().orc_fit_batch(C.byref(csr), C.byref(opts), C.byref(outs), int(n_threads))
    if rc != 0:
        raise RuntimeError(f"oracle fit failed: {rc}")
    return res


def finalize_batch(batch, model, pso_params, pso_cost=None, per_model_chi2=None, svi_mu=None, svi_log_sigma=None,
                   svi_elbo=None, method=abi.METHOD_SVI, n_threads=0) -> abi.FitResult:
    """finalize_parametric_from_gpu / finalize_*_with_gpu_svi over a batch
    (src/parametric.rs:3126-3553), selection rows as abi.selection_struct."""
    keep = []
    csr = abi.csr_struct(batch, keep)
    sel = abi.selection_struct(batch.n_bands, model, pso_params, pso_cost, per_model_chi2, svi_mu, svi_log_sigma,
                               svi_elbo, keep)
    res = abi.FitResult(batch.n_bands)
    outs = res.as_struct()
    rc = lib().orc_finalize_batch(C.byref(csr), sel.model, sel.pso_params, sel.pso_cost, sel.per_model_chi2,
                                  sel.svi_mu, sel.svi_log_sigma, sel.svi_elbo, int(method), C.byref(outs),
                                  int(n_threads))
    if rc != 0:
        raise RuntimeError(f"oracle finalize failed: {rc}")
    return res


def pso_stats(reset=True):
    out = np.zeros(4, np.int64)
    lib().orc_pso_stats(_p(out), int(reset))
    return dict(runs=int(out[0]), iters=int(out[1]), gbest_changes=int(out[2]), evals=int(out[3]))


def max_threads() -> int:
    return int(lib().orc_max_threads())


# --- the reference's GPU kernels (cuda/models.cu, cuda/svi.cu) --------------
def metzger_at_obs(params, t: float) -> float:
    """MetzgerKN at one observation as the reference's GPU kernels evaluate it
    (cuda/models_device.h:376-456)."""
    p = np.ascontiguousarray(params, np.float64)
    return float(lib().orc_metzger_at_obs(_p(p), float(t)))


def _gpu_band(band: Band):
    up = np.ascontiguousarray(band.up.astype(np.int32))
    return up, (_p(band.t), _p(band.f), _p(band.var), _p(up), _p(band.uf), band.n)


def gpu_pso_cost(model: int, band: Band, positions) -> np.ndarray:
    """batch_pso_cost (cuda/models.cu:516-584) of each row of ``positions``."""
    P = np.ascontiguousarray(np.atleast_2d(positions), np.float64)
    out = np.zeros(P.shape[0])
    up, args = _gpu_band(band)
    assert lib().orc_gpu_pso_cost(int(model), *args, _p(P), P.shape[0], P.shape[1], _p(out)) == 0
    return out


def gpu_mb_cost(band: Band, positions, k: int) -> np.ndarray:
    """batch_pso_cost_multi_bazin (cuda/models.cu:318-362), K = k, rows padded."""
    P = np.ascontiguousarray(np.atleast_2d(positions), np.float64)
    out = np.zeros(P.shape[0])
    up, args = _gpu_band(band)
    assert lib().orc_gpu_mb_cost(*args, _p(P), P.shape[0], P.shape[1], int(k), _p(out)) == 0
    return out


def gpu_svi_fit(model: int, band: Band, init, prior_c, prior_w, src: int, n_steps=1000, n_samples=4, lr=0.01):
    """batch_svi_fit (cuda/svi.cu:48-330) of one source whose index (its
    noise seed) is ``src``: (mu, log_sigma, elbo, steps)."""
    npar = abi.N_PARAMS[model]
    ini = np.ascontiguousarray(init[:npar], np.float64)
    pc = np.ascontiguousarray(prior_c[:npar], np.float64)
    pw = np.ascontiguousarray(prior_w[:npar], np.float64)
    mu, ls, elbo = np.zeros(npar), np.zeros(npar), np.zeros(1)
    up, args = _gpu_band(band)
    steps = lib().orc_gpu_svi_fit(int(model), *args, _p(ini), npar, abi.SE_IDX[model], _p(pc), _p(pw), int(n_steps),
                                  int(n_samples), float(lr), int(src), _p(mu), _p(ls), _p(elbo))
    assert steps >= 0
    return mu, ls, float(elbo[0]), steps


def set_laplace_step(step: float = 1e-4) -> None:
    """The relative finite-difference step of the oracle's Laplace Hessian
    (the reference's 1e-4, restored by the default).  A test hook: it measures
    how far the reference's own log sigma depends on the step."""
    lib().orc_set_laplace_step(float(step))


def set_cost_perturbation(rel: float, salt: int = 0, grad_rel: float = 0.0) -> None:
    """Perturb every swarm / polish / MultiBazin / joint multi-band cost of the oracle by +-rel
    and each polish gradient component by +-grad_rel (a hash of the parameter
    vector, the component and `salt` picks the signs); 0 restores the exact
    arithmetic.  A test hook: it measures how far the reference's own results
    move under rounding-sized changes of its costs and gradients."""
    lib().orc_set_cost_perturbation(float(rel), int(salt), float(grad_rel))


def set_position_perturbation(rel: float, salt: int = 0) -> None:
    """Scale every new interior swarm position component of the oracle by
    1 +- rel (a hash of the value, component, particle, iteration and `salt`
    picks the sign); 0 restores the exact arithmetic.  A test hook: it
    measures how far the reference's own results move when its swarm
    trajectories change by a rounding."""
    lib().orc_set_position_perturbation(float(rel), int(salt))

