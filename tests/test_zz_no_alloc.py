"""GPU test of lcf_band_cost_static, the allocation-free likelihood entry point.

Callers that cannot call cudaMalloc (a framework that owns all device memory
through its own pool, an embedding where the library must not allocate) pass
device buffers they already hold; the library's scratch for this call is a
fixed static device array.  The test calls it through the C ABI twice in a
row, on different bands and models (MetzgerKN, whose cost uses the scratch
for its interpolation buffer, and Bazin), and checks each result against the
existing entry point lcf_band_cost within the likelihood tolerance of the
parity tests.  It also checks a band with NaN times right after a different
band (every record slot must be rewritten by the call that reads it), the
capacity edge (2048 observations, 512 parameter vectors) against the FP64
oracle, and that the device's free memory does not change across calls.  It
runs alone in a fresh process as well as after the others.
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


def _edge_band(n=2048, seed=3):
    """A synthetic Bazin-shaped band of exactly n observations, peak-normalised."""
    rng = np.random.default_rng(seed)
    t = np.sort(rng.uniform(0.0, 300.0, n))
    F = 50.0 + 1000.0 * np.exp(-(t - 60.0) / 40.0) / (1.0 + np.exp(-(t - 60.0) / 5.0))
    e = 0.05 * np.abs(F) + 5.0
    f = F + rng.normal(0.0, e)
    peak = f.max()
    up = ((e > 0) & (f / e < 3.0)).astype(np.uint8)
    return t, f / peak, (e / peak) ** 2 + 1e-10, up, 3.0 * e / peak


@pytest.mark.parametrize("model", [0, 7])
def test_static_band_cost_at_capacity_matches_oracle(setup, oracle, model):
    """2048 observations x 512 parameter vectors: the whole static array is in
    use (MetzgerKN's per-lane interpolation buffer fills it).  Bazin is held
    to the likelihood criterion, 1e-5 of the FP64 cost below 1e6; MetzgerKN to
    the statistical bound of its Euler integration (median 1e-5, p90 1e-3),
    and to the allocating entry point, which runs the same FP32 arithmetic."""
    L, ctx = setup
    band = _edge_band()
    rng = np.random.default_rng(11 + model)
    P = rng.uniform(LO[model], HI[model], (512, len(LO[model])))
    if model == 0:
        P[:256, 2] = rng.uniform(0.0, 200.0, 256)  # t0 inside the span
    got = _static_cost(L, model, band, P)
    ob = oracle.Band.__new__(oracle.Band)
    ob.t, ob.f, ob.var, ob.up, ob.uf = [np.ascontiguousarray(a) for a in band]
    ref = oracle.band_cost(model, ob, P, with_prior=True)
    assert np.array_equal(got >= 1e98, ref >= 1e98)
    fin = ref < 1e98
    rel = np.abs(got[fin] - ref[fin]) / np.maximum(np.abs(ref[fin]), 1.0)
    if model == 0:
        assert rel[np.abs(ref[fin]) < 1e6].max(initial=0.0) < 1e-5
    else:
        assert np.median(rel) < 1e-5 and np.percentile(rel, 90) < 1e-3
        alloc = ctx.band_cost(model, *band, P, with_prior=True)
        fa = np.isfinite(alloc)
        assert np.allclose(got[fa], alloc[fa], rtol=1e-5, atol=0.0)


def test_static_band_cost_nan_times_after_another_band(setup):
    """A band whose times include NaN, right after a call on a different band
    of the same length: NaN times rank after all others, so every record slot
    is rewritten, and the costs equal the allocating entry point's (which
    orders NaN times the same way)."""
    L, ctx = setup
    first = _edge_band(300, seed=5)
    second = [a.copy() for a in _edge_band(300, seed=6)]
    second[0][[3, 150, 151]] = np.nan
    rng = np.random.default_rng(2)
    P = rng.uniform(LO[0], HI[0], (64, 6))
    P[:, 2] = rng.uniform(0.0, 200.0, 64)
    _static_cost(L, 0, first, P)
    got = _static_cost(L, 0, second, P)
    ref = ctx.band_cost(0, *second, P, with_prior=True)
    assert np.array_equal(got, ref)


def test_static_band_cost_allocates_nothing(setup):
    """Two calls after the first one leave the device's free memory and the
    torch caching allocator's reservation unchanged."""
    import torch
    L, _ = setup
    band = _edge_band(500, seed=9)
    rng = np.random.default_rng(4)
    P = rng.uniform(LO[7], HI[7], (200, 5))
    dev = [torch.as_tensor(np.ascontiguousarray(a), device="cuda") for a in band]
    p = torch.as_tensor(P, device="cuda")
    out = torch.zeros(200, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream

    def call():
        rc = L.lcf_band_cost_static(0, 7, *[x.data_ptr() for x in dev], 500, p.data_ptr(), 200, 1,
                                    out.data_ptr(), stream)
        assert rc == 0
        torch.cuda.synchronize()

    call()
    free0, _ = torch.cuda.mem_get_info()
    res0 = torch.cuda.memory_reserved()
    call()
    call()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0 and torch.cuda.memory_reserved() == res0
