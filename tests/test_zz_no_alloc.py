"""GPU test of lcf_band_cost_static, the allocation-free likelihood entry point.

Callers that cannot call cudaMalloc (a framework that owns all device memory
through its own pool, an embedding where the library must not allocate) pass
device buffers they already hold; the library's scratch for this call is a
fixed static device array.  The test calls it through the C ABI twice in a
row, on different bands and models (MetzgerKN, whose cost uses the scratch
for its interpolation buffer, and Bazin), and checks each result against the
existing entry point lcf_band_cost within the likelihood tolerance of the
parity tests.  It runs alone in a fresh process as well as after the others.
"""
import ctypes

import numpy as np
import pytest

from lightcurve_fitting_gb300 import abi, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from lightcurve_fitting_gb300 import build
    build.build()
    from lightcurve_fitting_gb300.lib import Context, load
    L = load()
    L.lcf_band_cost_static.argtypes = [ctypes.c_int, ctypes.c_int] + [ctypes.c_void_p] * 5 + [
        ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    ctx = Context(0)
    yield L, ctx
    ctx.close()


def _band(batch, s, b):
    t, f, e = batch.bands_of(s)[b]
    peak = f.max()
    fe = e / peak
    up = ((e > 0) & (f / e < 3.0)).astype(np.uint8)
    return t, f / peak, fe ** 2 + 1e-10, up, 3.0 * e / peak


def _static_cost(L, model, band, params, with_prior=True):
    import torch
    dev = [torch.as_tensor(np.ascontiguousarray(a), device="cuda") for a in band]
    p = torch.as_tensor(np.ascontiguousarray(params, np.float64), device="cuda")
    out = torch.full((params.shape[0],), float("nan"), dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rc = L.lcf_band_cost_static(0, model, *[x.data_ptr() for x in dev], band[0].size, p.data_ptr(),
                                params.shape[0], int(with_prior), out.data_ptr(), stream)
    assert rc == 0, rc
    torch.cuda.synchronize()
    return out.cpu().numpy()


LO = {0: [-3.0, -0.3, -100.0, -2.0, -2.0, -5.0], 7: [-3.0, -2.0, -1.0, -2.0, -5.0]}
HI = {0: [3.0, 0.3, 100.0, 5.0, 6.0, 0.0], 7: [-0.5, -0.5, 2.0, 1.0, 0.0]}


@pytest.mark.parametrize("model", [7, 0])
def test_static_band_cost_matches_allocating_entry_point_twice(setup, model):
    L, ctx = setup
    batch = synth.config_uneven(6, seed=77)
    rng = np.random.default_rng(5 + model)
    for call, (s, b) in enumerate([(1, 0), (4, 2)]):  # two calls in a row, different bands
        band = _band(batch, s, b)
        P = rng.uniform(LO[model], HI[model], (100 + 37 * call, len(LO[model])))
        got = _static_cost(L, model, band, P)
        ref = ctx.band_cost(model, *band, P, with_prior=True)
        assert np.all(np.isfinite(got) == np.isfinite(ref))
        fin = np.isfinite(ref)
        assert np.allclose(got[fin], ref[fin], rtol=1e-5, atol=0.0), call


def test_static_band_cost_rejects_sizes_beyond_capacity(setup):
    L, _ = setup
    import torch
    big = torch.zeros(4096, dtype=torch.float64, device="cuda")
    up = torch.zeros(4096, dtype=torch.uint8, device="cuda")
    p = torch.zeros(6, dtype=torch.float64, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    rc = L.lcf_band_cost_static(0, 0, big.data_ptr(), big.data_ptr(), big.data_ptr(), up.data_ptr(),
                                big.data_ptr(), 4096, p.data_ptr(), 1, 1, out.data_ptr(), None)
    assert rc == -6  # LCF_E_CAPACITY: more than 2048 observations
    rc = L.lcf_band_cost_static(0, 0, big.data_ptr(), big.data_ptr(), big.data_ptr(), up.data_ptr(),
                                big.data_ptr(), 100, p.data_ptr(), 513, 1, out.data_ptr(), None)
    assert rc == -6  # more than 512 parameter vectors
