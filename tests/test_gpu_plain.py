"""GPU tests of the plain FP64 form (lcf_fit_plain_device), the baseline the
fused pipeline is measured against.

The plain form moves every particle of an iteration with the previous
iteration's global best (synchronous PSO), where the reference's CPU loop
updates the best after each particle, so its swarms follow other trajectories
than the oracle's; after the L-BFGS polish both land in the same optimum for
most bands.  Its outputs are checked against the oracle on that basis:
identical fitted bands and ranks, the selected model for >= 85 % of bands,
per-model polished chi2 with a median relative gap below 1e-3, and finite SVI
posteriors.
"""
import numpy as np
import pytest

from lightcurve_fitting_gb300 import abi, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from lightcurve_fitting_gb300 import build
    build.build()
    from lightcurve_fitting_gb300.lib import Context
    c = Context(0)
    yield c
    c.close()


def _device(batch):
    import torch
    d = {
        "times": torch.from_numpy(batch.times).cuda(),
        "flux": torch.from_numpy(batch.flux).cuda(),
        "flux_err": torch.from_numpy(batch.flux_err).cuda(),
        "band_obs_offsets": torch.from_numpy(batch.band_obs_offsets).cuda(),
        "source_band_offsets": torch.from_numpy(batch.source_band_offsets).cuda(),
    }
    return d, {k: v.data_ptr() for k, v in d.items()}


def test_plain_form_selects_like_the_oracle(ctx, oracle):
    batch = synth.config_uneven(16, seed=31)
    keep, ptrs = _device(batch)
    ctx.fit_plain_device(ptrs, batch.n_sources, batch.n_bands, fit_all_models=True)
    res = ctx.download(batch.n_bands)
    ref = oracle.fit_batch(batch, fit_all_models=True, method=abi.METHOD_SVI, run_multi_bazin=False)
    fitted = ref.model >= 0
    assert np.array_equal(res.model >= 0, fitted)
    assert np.array_equal(res.rank, ref.rank)
    agree = (res.model[fitted] == ref.model[fitted]).mean()
    assert agree >= 0.85, agree
    a, b = res.per_model_chi2[fitted], ref.per_model_chi2[fitted]
    ok = np.isfinite(a) & np.isfinite(b)
    rel = (a[ok] - b[ok]) / np.maximum(np.abs(b[ok]), 1.0)
    assert np.median(np.abs(rel)) < 1e-3, np.median(np.abs(rel))
    np_sel = np.array([abi.N_PARAMS[m] for m in res.model[fitted]])
    mu = res.svi_mu[fitted]
    assert all(np.isfinite(mu[i, :k]).all() for i, k in enumerate(np_sel))
    assert np.isnan(res.mag_chi2).all() and (res.mb_best_k == 0).all()
    st = ctx.stats()
    assert st["kernel_launches"] == 1 + 8 + 8 + 1 + 8


def test_plain_form_bazin_gate(ctx):
    """fit_all_models = false: bands whose polished Bazin cost is below 2 keep
    Bazin and fit nothing else (src/parametric.rs:1862)."""
    batch = synth.config_basic(8, seed=3)
    keep, ptrs = _device(batch)
    ctx.fit_plain_device(ptrs, batch.n_sources, batch.n_bands, fit_all_models=False)
    res = ctx.download(batch.n_bands)
    fitted = res.model >= 0
    assert fitted.any()
    bz = res.per_model_chi2[:, 0]
    good = fitted & (bz < 2.0)
    others = res.per_model_chi2[:, 1:]
    assert np.isnan(others[good]).all()
    assert (res.model[good] == 0).all()
    assert np.isfinite(others[fitted & (bz >= 2.0)]).any(axis=1).all()


def test_plain_form_rejects_laplace(ctx):
    import ctypes as C
    batch = synth.config_basic(2, seed=1)
    keep, ptrs = _device(batch)
    csr = abi.BandsCSR()
    csr.n_sources, csr.n_bands = batch.n_sources, batch.n_bands
    csr.source_band_offsets = ptrs["source_band_offsets"]
    csr.band_obs_offsets = ptrs["band_obs_offsets"]
    csr.times, csr.flux, csr.flux_err = ptrs["times"], ptrs["flux"], ptrs["flux_err"]
    opts = abi.options(True, abi.METHOD_LAPLACE, -1, False)
    rc = ctx.L.lcf_fit_plain_device(ctx.h, C.byref(csr), C.byref(opts))
    assert rc == -5  # LCF_E_UNSUPPORTED
