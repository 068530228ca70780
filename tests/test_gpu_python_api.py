"""GPU tests of the Python mirror's model evaluation and joint multi-band
entry (python/src/lib.rs:257-269, 316-326)."""
import numpy as np
import pytest

from lightcurve_fitting_gb300 import abi, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from lightcurve_fitting_gb300 import build
    build.build()


PARAMS = {
    0: [0.3, 0.05, 12.0, 1.2, 3.1, -3.0],
    1: [0.1, 0.01, 2.5, 8.0, 1.0, 3.0, -3.0],
    2: [0.2, 0.1, 10.0, 1.0, 2.0, 1.5, -3.0],
    3: [0.1, 5.0, 2.3, 0.5, -3.0],
    4: [0.1, 5.0, 3.0, 2.3, -3.0],
    5: [0.1, 5.0, 0.5, 1.0, -3.0],
    6: [0.1, 5.0, 1.0, 0.8, 2.0, -3.0],
    7: [-1.75, -1.25, 0.5, -0.5, -3.0],
}


@pytest.mark.parametrize("m", range(8))
def test_eval_model_matches_the_oracle(gpu, oracle, m):
    """eval_model_flux through the drop-in kernels against the FP64 oracle, at
    the reference's own tolerances (tests/test_gpu.rs: 1e-10 absolute for
    Bazin, 1e-8 relative for the others); MetzgerKN's Euler sweep amplifies
    last-bit libm differences, so its median is held to 1e-6."""
    from lightcurve_fitting_gb300 import parametric
    t = np.concatenate([np.linspace(-20.0, 120.0, 57), [3.0, -1.0, 40.0]])  # unsorted tail
    got = np.array(parametric.eval_model(abi.MODEL_NAMES[m], PARAMS[m], t))
    ref = oracle.eval_model(m, np.array(PARAMS[m]), t)
    if m == 7:
        rel = np.abs(got - ref) / np.maximum(np.abs(ref), 1e-12)
        assert np.median(rel) < 1e-6, rel
    elif m == 0:
        assert np.max(np.abs(got - ref)) < 1e-10
    else:
        assert np.all(np.abs(got - ref) <= 1e-8 * np.maximum(np.abs(ref), 1e-10))


def _same(a, b):
    """Deep equality of result dicts with NaN equal to NaN (a MultiBazin
    result holds NaN for the K it did not fit)."""
    if isinstance(a, dict):
        return isinstance(b, dict) and a.keys() == b.keys() and all(_same(a[k], b[k]) for k in a)
    if isinstance(a, (list, tuple)):
        return isinstance(b, (list, tuple)) and len(a) == len(b) and all(_same(x, y) for x, y in zip(a, b))
    if isinstance(a, float) and isinstance(b, float) and np.isnan(a) and np.isnan(b):
        return True
    return a == b


def test_fit_parametric_multiband_is_the_joint_branch(gpu):
    """fit_parametric_multiband on a 3-band source gives what fit_parametric
    (fit_all_models=False) gives for it: the joint Villar fit."""
    from lightcurve_fitting_gb300 import parametric
    batch = synth.config_basic(1, seed=97)
    bands = {"gri"[k]: {"times": list(t), "values": list(f), "errors": list(e)}
             for k, (t, f, e) in enumerate(batch.bands_of(0))}
    a = parametric.fit_parametric_multiband(bands, method="laplace")
    b = parametric.fit_parametric(bands, fit_all_models=False, method="laplace")
    assert _same(a, b) and len(a) == 3
    assert all(r["model"] == "Villar" for r in a)
