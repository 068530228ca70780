"""Edge cases of the fused fit, through the C ABI against the oracle:
empty bands, one- to four-point bands, a source without bands, a source whose
only non-empty band is short (tests/ragged.py); an empty batch; and the joint
multi-band branch's limit of six bands with data per source (the reference
has none; the GPU reports LCF_E_UNSUPPORTED and the context stays usable)."""
import numpy as np
import pytest

from lightcurve_fitting_gb300 import abi, synth

import ragged

pytestmark = pytest.mark.gpu

KW = {
    "svi": dict(fit_all_models=True, method=abi.METHOD_SVI, run_multi_bazin=True),
    "laplace": dict(fit_all_models=True, method=abi.METHOD_LAPLACE, run_multi_bazin=True),
    "joint": dict(fit_all_models=False, method=abi.METHOD_LAPLACE, run_multi_bazin=True, joint_multiband=True),
}


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


@pytest.mark.parametrize("mode", list(KW))
def test_ragged_batch_matches_oracle(ctx, oracle, mode):
    """The same bands fitted and skipped, the same ranks and counts, MultiBazin
    on the same bands (rank 0 with >= 5 points), finite results for every
    fitted band, and on the bands of >= 12 points the oracle's model (a band
    of one to four points is fitted too, but many models fit it exactly)."""
    b = ragged.batch()
    g = ctx.fit_batch(b, **KW[mode])
    r = oracle.fit_batch(b, **KW[mode])
    assert np.array_equal(g.n_obs, r.n_obs) and np.array_equal(g.rank, r.rank)
    assert np.array_equal(g.model >= 0, r.model >= 0)
    assert np.array_equal(g.mb_best_k > 0, r.mb_best_k > 0)
    fitted = r.model >= 0
    assert fitted.sum() == 15 and not fitted[np.diff(b.band_obs_offsets) == 0].any()
    for name in ("pso_chi2", "svi_elbo"):
        assert np.all(np.isfinite(getattr(g, name)[fitted])), name
    k = abi.N_PARAMS
    for i in np.flatnonzero(fitted):
        assert np.all(np.isfinite(g.svi_mu[i, :k[g.model[i]]])), i
    long = fitted & (r.n_obs >= 12)
    if mode == "joint":
        # a source with two or more bands of data is the joint Villar fit
        assert np.array_equal(g.model[fitted] == 1, r.model[fitted] == 1)
    else:
        assert np.sum(g.model[long] != r.model[long]) <= 1, (g.model[long], r.model[long])


def test_empty_batch(ctx):
    empty = synth.PhotometryBatch(np.zeros(0), np.zeros(0), np.zeros(0), np.zeros(1, np.int64),
                                  np.zeros(1, np.int32), np.zeros(0, np.int32), "empty")
    for kw in KW.values():
        res = ctx.fit_batch(empty, **kw)
        assert res.model.size == 0


def test_joint_band_limit_is_reported_and_the_context_recovers(ctx):
    from lightcurve_fitting_gb300.lib import LcfError
    base = synth.config_basic(3, seed=43)
    bands = [base.bands_of(s)[k] for s in range(3) for k in range(3)][:7]
    t, f, e = (np.concatenate([x[i] for x in bands]) for i in range(3))
    bo = np.concatenate([[0], np.cumsum([len(x[0]) for x in bands])]).astype(np.int64)
    seven = synth.PhotometryBatch(t, f, e, bo, np.array([0, 7], np.int32), np.zeros(1, np.int32), "seven")
    with pytest.raises(LcfError):
        ctx.fit_batch(seven, **KW["joint"])
    res = ctx.fit_batch(seven, **KW["laplace"])  # the per-band path has no limit
    assert np.all(res.model >= 0)
    again = ctx.fit_batch(base, **KW["joint"])
    assert np.all(again.model == 1)
