"""The metric's own path against the oracle: fit_parametric_model with
fit_all_models = true, PSO model selection, SVI uncertainty (so the profile t0
search of each source's rank-0 band, src/parametric.rs:1767-1849 and
:3657-3661), the refinements and the MultiBazin fit (:904-1283), on the
uneven workload's generator, through the C ABI.

The reference's own results on this path move under perturbations of the
size of rounding.  With the oracle's costs perturbed by +-1e-7 (its test
hook, oracle.set_cost_perturbation) it changes the selected model of 7 of
600 bands, keeps only 93 % of posterior means within 0.1 sigma and 58 % /
72 % of the post-t0-search / polished costs within 1e-6; under +-1e-9 still
5 bands, 94 % and 74 % / 79 %.  Its polish is as sensitive to its gradient:
with each gradient component perturbed by +-1e-14 it changes 4 selections
and moves 10 % of the 4,800 polished costs by more than 1e-6 and 3 % by more
than 1e-3, each such polish ending on another local optimum (measured on
this workload, 200 sources).  The GPU's double-float sums differ from the
oracle's FP64 ones at that level: two GPU builds that differ only in the
summation order of the polish depart from the oracle in 37 and 43 band-
model polishes where the other build agrees with it, better and worse
about equally often.  Its MultiBazin fits do not move.  The criteria are
therefore stated against the oracle itself:
  * fitted bands and their ranks are identical;
  * >= 99 % of bands select the oracle's model (or as many as the perturbed
    oracles agree with the oracle, where that is fewer: 98.7 % on the basic
    workload's 300 bands, x86 and Arm); every disagreement is a near
    tie (BIC gap below 1e-3 of the best), a band where the reference is
    unstable (its choice, or its polished cost of one of the two models,
    moves under one of the perturbations: +-1e-7 with two sign patterns,
    +-1e-9, and +-1e-12 or +-1e-14 on the gradient), or a band where the GPU's polish
    of one of the two models ended on another local optimum (cost more than
    1e-4 away); and there are no more disagreements that are not near ties
    than the perturbed oracles have with the oracle.  The oracle's own
    choice can differ between hosts: on this workload it picks Afterglow for
    one band on x86 and Tde on Arm, whose libm rounds differently;
  * the reported cost of the selected model (the t0 search's on rank-0
    bands): median within 1e-9, and within 1e-6 at least as often as the
    perturbed oracle agrees with itself;
  * posterior means within 0.1 posterior sigma at least as often as the
    perturbed oracle's (less 2 points) and for >= 90 % of the bands;
  * MultiBazin: the same K for >= 98 % of rank-0 bands, and the cost of that K
    within 1e-4 for >= 95 % of them (measured 99 % / 97 %); and no more K
    changes or per-K cost departures (1e-4) than the oracle shows when its
    swarm positions are perturbed by 1e-15 (oracle.set_position_perturbation).
    Its swarms end the fit (no polish) and follow the reference's trajectory
    in double-float, ~2^-48 against FP64's 2^-53; the reference's K moves for
    2 of 200 sources when its positions move by 1e-16, 9-15 at 1e-15.
"""
import numpy as np
import pytest

from lightcurve_fitting_gb300 import abi, synth

from criteria import PERTURBATIONS, perturbed as _perturbed, selection_check, within as _within

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


def test_metric_path_matches_oracle(ctx, oracle):
    """200 uneven sources (600 bands), PSO + SVI with the t0 search and
    MultiBazin, against the FP64 oracle and the oracle's own sensitivity."""
    batch = synth.config_uneven(200, seed=123)
    kw = dict(fit_all_models=True, method=abi.METHOD_SVI, run_multi_bazin=True)
    res = ctx.fit_batch(batch, **kw)
    ref = oracle.fit_batch(batch, **kw)
    perts = [_perturbed(oracle, batch, *p, **kw) for p in PERTURBATIONS]
    pert = perts[0]
    frac, floor, bad, n, n_orc = selection_check(res, ref, perts)
    assert frac >= floor and not bad and n <= n_orc, (frac, floor, bad, n, n_orc)
    same = (ref.model >= 0) & (res.model == ref.model)
    same_p = same & (pert.model == ref.model)
    # the selected model's reported cost (post t0 search on rank-0 bands)
    c_gpu = _within(res.pso_chi2[same], ref.pso_chi2[same], 1e-6).mean()
    c_orc = _within(pert.pso_chi2[same_p], ref.pso_chi2[same_p], 1e-6).mean()
    rel = np.abs(res.pso_chi2[same] - ref.pso_chi2[same]) / np.maximum(np.abs(ref.pso_chi2[same]), 1e-12)
    assert np.median(rel) < 1e-9 and c_gpu >= c_orc, (np.median(rel), c_gpu, c_orc)
    r0 = same & (ref.rank == 0)
    c0_gpu = _within(res.pso_chi2[r0], ref.pso_chi2[r0], 1e-6).mean()
    c0_orc = _within(pert.pso_chi2[r0 & same_p], ref.pso_chi2[r0 & same_p], 1e-6).mean()
    assert c0_gpu >= c0_orc, (c0_gpu, c0_orc)
    # posterior means in the oracle's posterior sigma
    def zmax(r, mask):
        out = []
        for b in np.flatnonzero(mask):
            k = abi.N_PARAMS[ref.model[b]]
            out.append(np.max(np.abs(r.svi_mu[b, :k] - ref.svi_mu[b, :k]) / np.exp(ref.svi_log_sigma[b, :k])))
        return np.array(out)
    z_gpu, z_orc = zmax(res, same), zmax(pert, same_p)
    f_gpu, f_orc = np.mean(z_gpu < 0.1), np.mean(z_orc < 0.1)
    assert f_gpu >= 0.9 and f_gpu >= f_orc - 0.02, (f_gpu, f_orc)
    # MultiBazin on each source's rank-0 band
    mb = (ref.mb_best_k > 0) | (res.mb_best_k > 0)
    assert mb.sum() >= 150
    k_agree = np.mean(res.mb_best_k[mb] == ref.mb_best_k[mb])
    sk = mb & (res.mb_best_k == ref.mb_best_k)
    c_mb = _within(res.mb_cost[sk], ref.mb_cost[sk], 1e-4).mean()
    assert k_agree >= 0.98 and c_mb >= 0.95, (k_agree, c_mb)
    # ... and no more departures than the oracle's own under a rounding of its
    # swarm positions (1e-15; measured 9-15 K changes, 151-173 per-K costs)
    r0 = ref.rank == 0

    def mb_departures(r):
        a, b = r.mb_per_k_cost[r0], ref.mb_per_k_cost[r0]
        ok = np.isfinite(a) & np.isfinite(b)
        return int(np.sum(r.mb_best_k[r0] != ref.mb_best_k[r0])), int(np.sum(ok & ~_within(a, b, 1e-4)))

    k_gpu, c_gpu_mb = mb_departures(res)
    orc = []
    for salt in (0, 1):
        oracle.set_position_perturbation(1e-15, salt)
        try:
            orc.append(mb_departures(oracle.fit_batch(batch, **kw)))
        finally:
            oracle.set_position_perturbation(0.0)
    assert k_gpu <= min(o[0] for o in orc) and c_gpu_mb <= min(o[1] for o in orc), (k_gpu, c_gpu_mb, orc)
    # the reported BIC is the reference's 2 n cost + (4K + 2) ln n
    n = res.n_obs[sk]
    bic = 2.0 * res.mb_cost[sk] * n + (4 * res.mb_best_k[sk] + 2) * np.log(n)
    assert np.allclose(res.mb_bic[sk], bic, rtol=1e-9, atol=1e-9)


def test_basic_workload_laplace_matches_oracle(ctx, oracle):
    """The basic workload in full (100 sources x 3 bands x 30 points, Bazin
    generator), PSO + Laplace as the reference's CPU benchmark runs it: the
    same selection rule, and the polished costs to a median 1e-9."""
    batch = synth.config_basic(100, seed=21)
    kw = dict(fit_all_models=True, method=abi.METHOD_LAPLACE, run_multi_bazin=True)
    res = ctx.fit_batch(batch, **kw)
    ref = oracle.fit_batch(batch, **kw)
    perts = [_perturbed(oracle, batch, *p, **kw) for p in PERTURBATIONS]
    frac, floor, bad, n, n_orc = selection_check(res, ref, perts)
    assert frac >= floor and not bad and n <= max(n_orc, 1), (frac, floor, bad, n, n_orc)
    fitted = ref.model >= 0
    a, b = res.per_model_chi2[fitted], ref.per_model_chi2[fitted]
    ok = np.isfinite(a) & np.isfinite(b)
    rel = np.abs(a[ok] - b[ok]) / np.maximum(np.abs(b[ok]), 1e-12)
    assert np.median(rel) < 1e-9, np.median(rel)
