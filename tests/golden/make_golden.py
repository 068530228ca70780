"""Generate tests/golden/model_kats.npz from the reference's own code.

The reference crate (Rust) cannot be built here, but its device model header
cuda/models_device.h is plain FP64 C++ once `__device__` is defined away.
oracle/Makefile (target ``ref``) compiles it, through the harness
oracle/ref_pin/ref_models_host.cpp, into oracle/_ref/libref_models.so; this
script samples it and writes the outputs as golden vectors:

  * the forward-eval known-answer cases of tests/test_gpu.rs:10-47 (Bazin at
    t = 0, 0.5, ..., 49.5; the seven analytic models at t = -10 ... 39);
  * 32 random parameter vectors per analytic model (uniform in the PSO bounds
    of src/parametric.rs:1541-1579) at 32 random times, values and analytic
    gradients;
  * log_normal_cdf and erf_approx on a grid (src/parametric.rs:866-901 restate
    the same formulas as cuda/models_device.h:24-51);
  * MetzgerKN at single observations as the reference's GPU kernels evaluate
    it (lc_metzger_kn_at_single, cuda/models_device.h:376-456, reached
    through lc_eval_model_at(7, ...)): 32 parameter vectors in the MetzgerKN
    PSO box at 24 times each, with their own generator so the sets above are
    unchanged.

Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from lightcurve_fitting_gb300 import abi  # noqa: E402

REF_LIB = os.path.join(ROOT, "oracle", "_ref", "libref_models.so")

# PSO bounds of the analytic models, src/parametric.rs:1541-1579 (Bazin B
# bounds widened to +-1 so the golden set also covers the GPU variant's box)
BOUNDS = {
    0: ([-3.0, -1.0, -100.0, -2.0, -2.0, -5.0], [3.0, 1.0, 100.0, 5.0, 6.0, 0.0]),
    1: ([-1.5, -0.02, 1.0, -60.0, -1.0, 1.0, -6.0], [1.5, 0.05, 5.0, 40.0, 3.0, 5.5, 0.0]),
    2: ([-3.0, -1.0, -100.0, -2.0, -1.0, 0.5, -5.0], [3.0, 1.0, 100.0, 5.0, 6.0, 4.0, 0.0]),
    3: ([-3.0, -100.0, 0.5, -3.0, -5.0], [3.0, 100.0, 4.5, 3.0, 0.0]),
    4: ([-3.0, -100.0, 0.0, 0.5, -5.0], [3.0, 100.0, 6.0, 4.5, 0.0]),
    5: ([-3.0, -100.0, 0.1, -1.0, -5.0], [3.0, 100.0, 3.0, 4.0, 0.0]),
    6: ([-3.0, -100.0, -2.0, -2.0, 0.5, -5.0], [3.0, 100.0, 6.0, 3.0, 5.0, 0.0]),
}

# tests/test_gpu.rs:24-47
KAT_PARAMS = {
    0: [0.5, 0.1, 10.0, 1.0, 3.0, -3.0],
    1: [0.5, 0.01, 2.0, 10.0, 1.0, 3.0, -3.0],
    2: [0.5, 0.1, 5.0, 1.0, 3.0, 1.67, -3.0],
    3: [0.5, 5.0, 2.3, 0.0, -3.0],
    4: [0.5, 5.0, 3.0, 2.3, -3.0],
    5: [0.5, 5.0, 0.5, 1.0, -3.0],
    6: [0.5, 5.0, 2.0, 0.8, 2.2, -3.0],
}


def load_ref():
    if not os.path.exists(REF_LIB):
        subprocess.check_call(["make", "-C", os.path.join(ROOT, "oracle"), "ref"])
    L = C.CDLL(REF_LIB)
    L.ref_eval.argtypes = [C.c_int, C.c_void_p, C.c_double]
    L.ref_eval.restype = C.c_double
    L.ref_grad.argtypes = [C.c_int, C.c_void_p, C.c_double, C.c_void_p]
    L.ref_grad.restype = C.c_int
    L.ref_log_normal_cdf.argtypes = [C.c_double]
    L.ref_log_normal_cdf.restype = C.c_double
    L.ref_erf_approx.argtypes = [C.c_double]
    L.ref_erf_approx.restype = C.c_double
    return L


def main():
    L = load_ref()
    rng = np.random.default_rng(20261203)
    out = {}

    def ev(m, p, times):
        p = np.ascontiguousarray(p, np.float64)
        return np.array([L.ref_eval(m, p.ctypes.data, float(t)) for t in times])

    def gr(m, p, times):
        p = np.ascontiguousarray(p, np.float64)
        g = np.zeros((len(times), abi.N_PARAMS[m]))
        for i, t in enumerate(times):
            buf = np.zeros(abi.N_PARAMS[m])
            assert L.ref_grad(m, p.ctypes.data, float(t), buf.ctypes.data) == 1
            g[i] = buf
        return g

    # known-answer cases of tests/test_gpu.rs
    t_bazin = np.arange(100) * 0.5
    out["kat_bazin_t"] = t_bazin
    out["kat_bazin_p"] = np.array(KAT_PARAMS[0])
    out["kat_bazin_f"] = ev(0, KAT_PARAMS[0], t_bazin)
    t_all = np.arange(-10, 40, dtype=np.float64)
    out["kat_all_t"] = t_all
    for m, p in KAT_PARAMS.items():
        out[f"kat_m{m}_p"] = np.array(p)
        out[f"kat_m{m}_f"] = ev(m, p, t_all)
        out[f"kat_m{m}_g"] = gr(m, p, t_all)
    # random parameter points inside the PSO boxes
    for m, (lo, hi) in BOUNDS.items():
        lo, hi = np.array(lo), np.array(hi)
        P = rng.uniform(lo, hi, (32, lo.size))
        T = np.sort(rng.uniform(-50.0, 250.0, 32))
        out[f"rand_m{m}_p"] = P
        out[f"rand_m{m}_t"] = T
        out[f"rand_m{m}_f"] = np.stack([ev(m, p, T) for p in P])
        out[f"rand_m{m}_g"] = np.stack([gr(m, p, T) for p in P])
    x = np.concatenate([np.linspace(-40.0, 10.0, 501), [-30.0000001, -29.9999999, 8.0, 8.0000001]])
    out["lncdf_x"] = x
    out["lncdf_y"] = np.array([L.ref_log_normal_cdf(float(v)) for v in x])
    xe = np.linspace(-6.0, 6.0, 241)
    out["erf_x"] = xe
    out["erf_y"] = np.array([L.ref_erf_approx(float(v)) for v in xe])
    # MetzgerKN per observation (bounds src/parametric.rs:1576-1578)
    rng7 = np.random.default_rng(20261204)
    lo7, hi7 = np.array([-3.0, -2.0, -1.0, -2.0, -5.0]), np.array([-0.5, -0.5, 2.0, 1.0, 0.0])
    P7 = rng7.uniform(lo7, hi7, (32, 5))
    T7 = np.sort(np.concatenate([rng7.uniform(-5.0, 3.0, 8), rng7.uniform(3.0, 60.0, 16)]))
    out["single_m7_p"] = P7
    out["single_m7_t"] = T7
    out["single_m7_f"] = np.stack([ev(7, p, T7) for p in P7])
    path = os.path.join(HERE, "model_kats.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, sum(v.size for v in out.values()), "values")


if __name__ == "__main__":
    main()
