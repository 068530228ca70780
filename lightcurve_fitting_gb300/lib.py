"""ctypes binding of liblcf_gb300.so (the C ABI of include/lcf.h).

The library is built in-tree by ``lightcurve_fitting_gb300.build``.  There is
no fallback: if the shared library is missing or no CUDA device is visible,
``Context`` raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liblcf_gb300.so")

_lib = None


class LcfError(RuntimeError):
    pass


def load(path: str = LIB_PATH):
    """Load the shared library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise LcfError(f"{path} is missing: build it with `python -m lightcurve_fitting_gb300.build` "
                       "(or __graft_entry__.build())")
    L = C.CDLL(path)
    vp, i, d = C.c_void_p, C.c_int, C.c_double
    L.lcf_ctx_create.argtypes = [i, C.POINTER(vp)]
    L.lcf_ctx_destroy.argtypes = [vp]
    L.lcf_last_error.argtypes = [vp]
    L.lcf_last_error.restype = C.c_char_p
    L.lcf_last_stats.argtypes = [vp, C.POINTER(abi.FitStats)]
    L.lcf_fit_parametric_batch.argtypes = [vp, C.POINTER(abi.BandsCSR), C.POINTER(abi.FitOptions),
                                           C.POINTER(abi.FitOutputs)]
    L.lcf_fit_parametric_batch_async.argtypes = [vp, C.POINTER(abi.BandsCSR), C.POINTER(abi.FitOptions),
                                                 C.POINTER(abi.FitOutputs)]
    L.lcf_wait.argtypes = [vp, i]
    L.lcf_fit_parametric_device.argtypes = [vp, C.POINTER(abi.BandsCSR), C.POINTER(abi.FitOptions)]
    L.lcf_finalize_batch.argtypes = [vp, C.POINTER(abi.BandsCSR), C.POINTER(abi.PsoSelection), i,
                                     C.POINTER(abi.FitOutputs)]
    L.lcf_fit_plain_device.argtypes = [vp, C.POINTER(abi.BandsCSR), C.POINTER(abi.FitOptions)]
    L.lcf_download_outputs.argtypes = [vp, C.POINTER(abi.FitOutputs)]
    L.lcf_ctx_stream.argtypes = [vp]
    L.lcf_ctx_stream.restype = vp
    L.lcf_set_graph.argtypes = [vp, i]
    L.lcf_set_wait_bound.argtypes = [vp, i]
    L.lcf_band_cost.argtypes = [vp, i, vp, vp, vp, vp, vp, i, vp, i, i, vp]
    L.lcf_set_autotune.argtypes = [vp, i, i]
    L.lcf_set_multi_bazin_branch.argtypes = [vp, i]
    L.lcf_autotune_candidates.argtypes = [vp, vp]
    L.lcf_autotune_table.argtypes = [vp, vp, i]
    L.lcf_autotune_load.argtypes = [vp, vp, i]
    L.lcf_last_launch.argtypes = [vp, vp]
    L.lcf_svi_elbo_grad.argtypes = [vp, i, vp, vp, vp, vp, vp, i, vp, vp, i, vp, i, vp, vp, vp]
    L.lcf_probe_peaks.argtypes = [vp, vp]
    L.lcf_probe_fp64.argtypes = [vp, vp]
    L.lcf_probe_ff.argtypes = [vp, vp]
    L.lcf_debug_swarm_results.argtypes = [vp, vp, C.c_int64]
    for name in ["launch_bazin", "launch_villar", "launch_tde", "launch_arnett", "launch_magnetar",
                 "launch_shock_cooling", "launch_afterglow", "launch_metzger_kn"]:
        getattr(L, name).argtypes = [vp, vp, vp, i, i, i, i, i]
        getattr(L, name).restype = None
    L.launch_batch_pso_cost.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp, i, i, i, i, i, i]
    L.launch_batch_pso_cost.restype = None
    L.launch_batch_pso_cost_multi_bazin.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp, vp, i, i, i, i, i]
    L.launch_batch_pso_cost_multi_bazin.restype = None
    L.launch_batch_svi_fit.argtypes = [vp] * 15 + [i, i, i, i, d, i, i]
    L.launch_batch_svi_fit.restype = None
    _lib = L
    return L


EVAL_EXPORTS = ["launch_bazin", "launch_villar", "launch_tde", "launch_arnett", "launch_magnetar",
                "launch_shock_cooling", "launch_afterglow", "launch_metzger_kn"]


class Context:
    """A GPU context: one CUDA stream, device buffers and a captured graph."""

    def __init__(self, device: int = 0):
        self.L = load()
        h = C.c_void_p()
        rc = self.L.lcf_ctx_create(int(device), C.byref(h))
        if rc != 0:
            raise LcfError(f"lcf_ctx_create({device}) failed with status {rc} (no CUDA device?)")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.L.lcf_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int, what: str):
        if rc != 0:
            msg = self.L.lcf_last_error(self.h).decode(errors="replace")
            raise LcfError(f"{what} failed with status {rc}: {msg}")

    @property
    def stream(self) -> int:
        return int(self.L.lcf_ctx_stream(self.h) or 0)

    def set_wait_bound(self, polls: int):
        """Bound of the swarm kernel's staging wait, in polls (test hook: 0
        makes every wait expire; the fit then returns LCF_E_TIMEOUT)."""
        self._check(self.L.lcf_set_wait_bound(self.h, int(polls)), "lcf_set_wait_bound")

    def set_graph(self, enabled: bool):
        self._check(self.L.lcf_set_graph(self.h, int(bool(enabled))), "lcf_set_graph")

    def fit_batch(self, batch, fit_all_models=True, method=abi.METHOD_SVI, forced_model=-1,
                  run_multi_bazin=True, joint_multiband=False) -> abi.FitResult:
        """lcf_fit_parametric_batch over a PhotometryBatch (host arrays)."""
        keep = []
        csr = abi.csr_struct(batch, keep)
        opts = abi.options(fit_all_models, method, forced_model, run_multi_bazin, joint_multiband)
        res = abi.FitResult(batch.n_bands)
        outs = res.as_struct()
        self._check(self.L.lcf_fit_parametric_batch(self.h, C.byref(csr), C.byref(opts), C.byref(outs)),
                    "lcf_fit_parametric_batch")
        return res

    def fit_batch_async(self, batch, fit_all_models=True, method=abi.METHOD_SVI, forced_model=-1,
                        run_multi_bazin=True, joint_multiband=False) -> abi.FitResult:
        """lcf_fit_parametric_batch_async: queues the fit and returns its
        (not yet filled) result; wait() fills it."""
        keep = []
        csr = abi.csr_struct(batch, keep)
        opts = abi.options(fit_all_models, method, forced_model, run_multi_bazin, joint_multiband)
        res = abi.FitResult(batch.n_bands)
        outs = res.as_struct()
        self._check(self.L.lcf_fit_parametric_batch_async(self.h, C.byref(csr), C.byref(opts), C.byref(outs)),
                    "lcf_fit_parametric_batch_async")
        self._pending = (res, outs)  # the output arrays stay alive until wait()
        return res

    def wait(self, timeout_ms: int = -1) -> int:
        """lcf_wait: 0 once the pending fit is written, LCF_E_TIMEOUT (-4)
        while it runs; raises on the fit's own errors."""
        rc = self.L.lcf_wait(self.h, int(timeout_ms))
        if rc == abi.LCF_E_TIMEOUT and "not finished" in self.L.lcf_last_error(self.h).decode(errors="replace"):
            return rc
        self._pending = None
        self._check(rc, "lcf_wait")
        return rc

    def finalize_batch(self, batch, model, pso_params, pso_cost=None, per_model_chi2=None, svi_mu=None,
                       svi_log_sigma=None, svi_elbo=None, method=abi.METHOD_SVI) -> abi.FitResult:
        """lcf_finalize_batch: uncertainty (unless svi_mu / svi_log_sigma are
        given), refinements and magnitude chi2 of caller-selected fits."""
        keep = []
        csr = abi.csr_struct(batch, keep)
        sel = abi.selection_struct(batch.n_bands, model, pso_params, pso_cost, per_model_chi2, svi_mu,
                                   svi_log_sigma, svi_elbo, keep)
        res = abi.FitResult(batch.n_bands)
        outs = res.as_struct()
        self._check(self.L.lcf_finalize_batch(self.h, C.byref(csr), C.byref(sel), int(method), C.byref(outs)),
                    "lcf_finalize_batch")
        return res

    def fit_device(self, dev_ptrs: dict, n_sources: int, n_bands: int, fit_all_models=True,
                   method=abi.METHOD_SVI, forced_model=-1, run_multi_bazin=True, joint_multiband=False):
        """lcf_fit_parametric_device over device pointers (keys: times, flux,
        flux_err, band_obs_offsets, source_band_offsets)."""
        csr = abi.BandsCSR()
        csr.n_sources, csr.n_bands = n_sources, n_bands
        csr.source_band_offsets = dev_ptrs["source_band_offsets"]
        csr.band_obs_offsets = dev_ptrs["band_obs_offsets"]
        csr.times, csr.flux, csr.flux_err = dev_ptrs["times"], dev_ptrs["flux"], dev_ptrs["flux_err"]
        opts = abi.options(fit_all_models, method, forced_model, run_multi_bazin, joint_multiband)
        self._check(self.L.lcf_fit_parametric_device(self.h, C.byref(csr), C.byref(opts)),
                    "lcf_fit_parametric_device")

    def fit_plain_device(self, dev_ptrs: dict, n_sources: int, n_bands: int, fit_all_models=True, forced_model=-1):
        """lcf_fit_plain_device: the plain FP64 GPU form (PSO, L-BFGS,
        selection, SVI; one launch per model per stage, no graph)."""
        csr = abi.BandsCSR()
        csr.n_sources, csr.n_bands = n_sources, n_bands
        csr.source_band_offsets = dev_ptrs["source_band_offsets"]
        csr.band_obs_offsets = dev_ptrs["band_obs_offsets"]
        csr.times, csr.flux, csr.flux_err = dev_ptrs["times"], dev_ptrs["flux"], dev_ptrs["flux_err"]
        opts = abi.options(fit_all_models, abi.METHOD_SVI, forced_model, False)
        self._check(self.L.lcf_fit_plain_device(self.h, C.byref(csr), C.byref(opts)), "lcf_fit_plain_device")

    def download(self, n_bands: int) -> abi.FitResult:
        res = abi.FitResult(n_bands)
        outs = res.as_struct()
        self._check(self.L.lcf_download_outputs(self.h, C.byref(outs)), "lcf_download_outputs")
        return res

    def stats(self) -> dict:
        s = abi.FitStats()
        self._check(self.L.lcf_last_stats(self.h, C.byref(s)), "lcf_last_stats")
        out = {}
        for k, _ in abi.FitStats._fields_:
            v = getattr(s, k)
            out[k] = list(v) if hasattr(v, "__len__") else v
        return out

    def probe_peaks(self) -> dict:
        buf = np.zeros(2)
        self._check(self.L.lcf_probe_peaks(self.h, buf.ctypes.data), "lcf_probe_peaks")
        return {"fp32_tflops": float(buf[0]), "mufu_gops": float(buf[1])}

    def probe_fp64(self) -> dict:
        """FP64 ceilings of the polish: per-model observation-term evaluations
        per second (models 0..6) and the DFMA-chain FP64 TFLOP/s."""
        buf = np.zeros(9)
        self._check(self.L.lcf_probe_fp64(self.h, buf.ctypes.data), "lcf_probe_fp64")
        return {"obs_evals_per_s": [float(v) for v in buf[:8]], "fp64_tflops": float(buf[8])}

    def probe_ff(self) -> dict:
        """The polish's double-float observation term: per-model evaluations
        per second, and its largest disagreement with the FP64 term (overall,
        and per cost / gradient component) over 256 points per model."""
        buf = np.zeros(80)
        self._check(self.L.lcf_probe_ff(self.h, buf.ctypes.data), "lcf_probe_ff")
        return {"obs_evals_per_s": [float(v) for v in buf[:7]], "worst_rel": [float(v) for v in buf[7:14]],
                "worst_rel_by_component": buf[14:70].reshape(7, 8).tolist(),
                "points_in_range": [int(v) for v in buf[70:77]], "nonfinite_mismatch": int(buf[77])}

    def swarm_results(self, n_bands: int) -> np.ndarray:
        """Raw swarm results of the last fit: (44 * n_bands, 21) rows, see lcf.h."""
        out = np.zeros((44 * n_bands, 21))
        self._check(self.L.lcf_debug_swarm_results(self.h, out.ctypes.data, out.shape[0]),
                    "lcf_debug_swarm_results")
        return out

    def band_cost(self, model: int, times, flux, obs_var, is_upper, upper_flux, params, with_prior=True):
        """PsoCost::cost_from_slice for each row of ``params`` (FP32 kernel)."""
        t = np.ascontiguousarray(times, np.float64)
        f = np.ascontiguousarray(flux, np.float64)
        v = np.ascontiguousarray(obs_var, np.float64)
        u = np.ascontiguousarray(is_upper, np.uint8)
        uf = np.ascontiguousarray(upper_flux, np.float64)
        p = np.ascontiguousarray(np.atleast_2d(params), np.float64)
        out = np.zeros(p.shape[0])
        self._check(self.L.lcf_band_cost(self.h, int(model), t.ctypes.data, f.ctypes.data, v.ctypes.data,
                                         u.ctypes.data, uf.ctypes.data, t.size, p.ctypes.data, p.shape[0],
                                         int(bool(with_prior)), out.ctypes.data), "lcf_band_cost")
        return out

    def set_multi_bazin_branch(self, mode: int):
        """0: stages in sequence; 1 / 2: MultiBazin K = 2..4 on a second
        stream forked after the model-selection swarm / the selection."""
        self._check(self.L.lcf_set_multi_bazin_branch(self.h, int(mode)), "lcf_set_multi_bazin_branch")

    def set_autotune(self, mode: int = 1, forced_candidate: int = -1):
        """Online launch tuning per shape bucket (mode 1), off (0), or a pinned candidate."""
        self._check(self.L.lcf_set_autotune(self.h, int(mode), int(forced_candidate)), "lcf_set_autotune")

    def autotune_candidates(self) -> np.ndarray:
        """(n, 3): block, staging depth, resident blocks per SM of each candidate."""
        out = np.zeros(9, np.int32)
        n = self.L.lcf_autotune_candidates(self.h, out.ctypes.data)
        return out[:3 * n].reshape(n, 3)

    def autotune_table(self) -> np.ndarray:
        """(buckets, 6): bucket, chosen candidate (-1 while exploring), next, stage ms per candidate."""
        n = self.L.lcf_autotune_table(self.h, None, 0)
        rows = np.zeros((max(n, 1), 6))
        self.L.lcf_autotune_table(self.h, rows.ctypes.data, n)
        return rows[:n]

    def autotune_load(self, rows):
        r = np.ascontiguousarray(np.atleast_2d(rows), np.float64)
        self._check(self.L.lcf_autotune_load(self.h, r.ctypes.data, r.shape[0]), "lcf_autotune_load")

    def last_launch(self) -> dict:
        out = np.zeros(4, np.int32)
        self._check(self.L.lcf_last_launch(self.h, out.ctypes.data), "lcf_last_launch")
        return {"candidate": int(out[0]), "block": int(out[1]), "smem_obs": int(out[2]), "bucket": int(out[3])}

    def svi_elbo_grad(self, model: int, times, flux, obs_var, is_upper, upper_flux, prior_init, var_params, eps):
        """One SVI step's ELBO estimate and its gradient (the SVI kernel's
        adjoint) at each row of ``var_params`` = [mu, log_sigma] (n_points,
        2 np), with the standard-normal draws ``eps`` (n_points, n_samples,
        np).  Returns (elbo [n_points], grad [n_points, 2 np], flags
        [n_points]), as lcf_svi_elbo_grad."""
        npar = abi.N_PARAMS[model]
        t = np.ascontiguousarray(times, np.float64)
        f = np.ascontiguousarray(flux, np.float64)
        v = np.ascontiguousarray(obs_var, np.float64)
        u = np.ascontiguousarray(is_upper, np.uint8)
        uf = np.ascontiguousarray(upper_flux, np.float64)
        ini = np.ascontiguousarray(prior_init, np.float64)
        vpar = np.ascontiguousarray(np.atleast_2d(var_params), np.float64)
        n_points = vpar.shape[0]
        e = np.ascontiguousarray(eps, np.float64).reshape(n_points, -1, npar)
        if ini.size != npar or vpar.shape[1] != 2 * npar:
            raise LcfError(f"model {model}: prior_init needs {npar} values and var_params {2 * npar} columns")
        elbo = np.zeros(n_points)
        grad = np.zeros((n_points, 2 * npar))
        flags = np.zeros(n_points, np.int32)
        self._check(self.L.lcf_svi_elbo_grad(self.h, int(model), t.ctypes.data, f.ctypes.data, v.ctypes.data,
                                             u.ctypes.data, uf.ctypes.data, t.size, ini.ctypes.data,
                                             vpar.ctypes.data, n_points, e.ctypes.data, e.shape[1],
                                             elbo.ctypes.data, grad.ctypes.data, flags.ctypes.data),
                    "lcf_svi_elbo_grad")
        return elbo, grad, flags


_default = None


def default_context() -> Context:
    global _default
    if _default is None:
        _default = Context(0)
    return _default
