"""CPU tests of the FP64 oracle: pinned against the reference's own model
code (golden vectors from cuda/models_device.h), plus algorithm checks of the
restated third-party pieces (SmallRng stream, analytic gradients vs central
finite differences) and the structural properties the reference's own tests
assert (tests/test_parametric.rs)."""
import numpy as np
import pytest

from lightcurve_fitting_gb300 import abi, synth


def test_golden_kats_bazin(oracle, golden):
    # tests/test_gpu.rs:10-22 requires |gpu - cpu| < 1e-10
    f = oracle.eval_model(0, golden["kat_bazin_p"], golden["kat_bazin_t"])
    assert np.max(np.abs(f - golden["kat_bazin_f"])) < 1e-10


@pytest.mark.parametrize("m", range(7))
def test_golden_kats_all_models(oracle, golden, m):
    t = golden["kat_all_t"]
    f = oracle.eval_model(m, golden[f"kat_m{m}_p"], t)
    ref = golden[f"kat_m{m}_f"]
    # tests/test_gpu.rs:41-44: relative 1e-8
    assert np.all(np.abs(f - ref) <= 1e-8 * np.maximum(np.abs(ref), 1e-10))
    g = oracle.eval_grad(m, golden[f"kat_m{m}_p"], t)
    gr = golden[f"kat_m{m}_g"]
    assert np.allclose(g, gr, rtol=1e-9, atol=1e-12)


@pytest.mark.parametrize("m", range(7))
def test_golden_random_points(oracle, golden, m):
    P, T = golden[f"rand_m{m}_p"], golden[f"rand_m{m}_t"]
    F, G = golden[f"rand_m{m}_f"], golden[f"rand_m{m}_g"]
    for k in range(P.shape[0]):
        f = oracle.eval_model(m, P[k], T)
        same_nonfinite = ~np.isfinite(F[k])
        assert np.array_equal(~np.isfinite(f), same_nonfinite)
        ok = np.isfinite(F[k])
        assert np.allclose(f[ok], F[k][ok], rtol=1e-10, atol=1e-300)
        g = oracle.eval_grad(m, P[k], T)
        okg = np.isfinite(G[k])
        assert np.array_equal(np.isfinite(g), okg)
        assert np.allclose(g[okg], G[k][okg], rtol=1e-9, atol=1e-300)


def test_golden_log_normal_cdf_and_erf(oracle, golden):
    y = np.array([oracle.lib().orc_log_normal_cdf(float(x)) for x in golden["lncdf_x"]])
    assert np.allclose(y, golden["lncdf_y"], rtol=1e-13, atol=0)
    e = np.array([oracle.lib().orc_erf_approx(float(x)) for x in golden["erf_x"]])
    assert np.allclose(e, golden["erf_y"], rtol=1e-14, atol=1e-16)


def _xoshiro256pp(seed, n):
    """Independent pure-Python restatement of xoshiro256++ seeded through
    SplitMix64 (Blackman & Vigna), the algorithm of rand 0.9's SmallRng."""
    M = (1 << 64) - 1
    s, st = [], seed
    for _ in range(4):
        st = (st + 0x9E3779B97F4A7C15) & M
        z = st
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M
        s.append(z ^ (z >> 31))
    rotl = lambda x, k: ((x << k) | (x >> (64 - k))) & M
    out = []
    for _ in range(n):
        out.append((rotl((s[0] + s[3]) & M, 23) + s[0]) & M)
        t = (s[1] << 17) & M
        s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3]; s[2] ^= t
        s[3] = rotl(s[3], 45)
    return out


@pytest.mark.parametrize("seed", [0, 42, 137, 271])
def test_rng_stream_matches_independent_restatement(oracle, seed):
    got = oracle.rng_stream(seed, 200)
    ref = np.array(_xoshiro256pp(seed, 200), dtype=np.uint64)
    assert np.array_equal(got, ref)
    f = oracle.rng_f64(seed, 200)
    assert np.array_equal(f, (ref >> np.uint64(11)).astype(np.float64) * 2.0 ** -53)
    assert np.all((f >= 0) & (f < 1))


def _band(seed=1, src=0, b=0):
    batch = synth.config_basic(3, seed=seed)
    t, f, e = batch.bands_of(src)[b]
    from oracle.oracle import Band
    return Band(t, f, e)


@pytest.mark.parametrize("m", range(7))
@pytest.mark.parametrize("with_upper", [False, True])
def test_cost_gradient_vs_central_fd(oracle, m, with_upper):
    # PsoCost::gradient (src/parametric.rs:1387-1445) is exact for detections;
    # for upper limits it divides the exact Gaussian pdf by the A&S 7.1.26
    # CDF, which is not the derivative of the approximated log-CDF in the
    # cost, so only agreement to ~1e-2 holds there.
    band = _band()
    if not with_upper:
        band.up[:] = 0
    rtol = 1e-2 if with_upper else 2e-5
    rng = np.random.default_rng(m)
    lo, hi = [np.array(v) for v in _bounds(m)]
    checked = 0
    for _ in range(20):
        p = rng.uniform(lo, hi)
        p[abi.SE_IDX[m]] = -2.0
        c0 = oracle.band_cost(m, band, p, with_prior=False)[0]
        if not np.isfinite(c0) or c0 > 1e6:
            continue
        g = oracle.band_cost_grad(m, band, p)
        if with_upper:
            pred = oracle.eval_model(m, p, band.t)
            z = (band.uf - pred) / np.sqrt(band.var + np.exp(2 * p[abi.SE_IDX[m]]))
            if np.any(band.up.astype(bool) & (z < -5.0)):
                # an upper limit violated by > 5 sigma: the reference's FP64 CDF
                # loses its digits (1 - (1 - P) with P < 1e-7) and, beyond
                # ~8.3 sigma, rounds to 0 and is floored at 1e-300
                continue
        fd = np.zeros_like(g)
        for j in range(p.size):
            h = 1e-6 * max(abs(p[j]), 1.0)
            pp, pm = p.copy(), p.copy()
            pp[j] += h
            pm[j] -= h
            fd[j] = (oracle.band_cost(m, band, pp, False)[0] - oracle.band_cost(m, band, pm, False)[0]) / (2 * h)
        assert np.allclose(g, fd, rtol=rtol, atol=rtol * 1e-2 * max(1.0, np.abs(fd).max())), (m, p, g, fd)
        checked += 1
    assert checked >= 3


def _bounds(m):
    return {
        0: ([-3.0, -0.3, -100.0, -2.0, -2.0, -5.0], [3.0, 0.3, 100.0, 5.0, 6.0, 0.0]),
        1: ([-1.5, -0.02, 1.0, -60.0, -1.0, 1.0, -6.0], [1.5, 0.05, 5.0, 40.0, 3.0, 5.5, 0.0]),
        2: ([-3.0, -1.0, -100.0, -2.0, -1.0, 0.5, -5.0], [3.0, 1.0, 100.0, 5.0, 6.0, 4.0, 0.0]),
        3: ([-3.0, -100.0, 0.5, -3.0, -5.0], [3.0, 100.0, 4.5, 3.0, 0.0]),
        4: ([-3.0, -100.0, 0.0, 0.5, -5.0], [3.0, 100.0, 6.0, 4.5, 0.0]),
        5: ([-3.0, -100.0, 0.1, -1.0, -5.0], [3.0, 100.0, 3.0, 4.0, 0.0]),
        6: ([-3.0, -100.0, -2.0, -2.0, 0.5, -5.0], [3.0, 100.0, 6.0, 3.0, 5.0, 0.0]),
        7: ([-3.0, -2.0, -1.0, -2.0, -5.0], [-0.5, -0.5, 2.0, 1.0, 0.0]),
    }[m]


def test_metzger_eval_properties(oracle):
    t = np.linspace(0, 30, 40)
    f = oracle.eval_model(7, [-2.0, -0.7, 0.5, -0.5, -3.0], t)
    assert np.all(np.isfinite(f)) and f.max() <= 1.0 + 1e-12 and f.min() >= 0.0
    # t0 after every observation: all zeros (src/parametric.rs:552-554)
    assert np.all(oracle.eval_model(7, [-2.0, -0.7, 0.5, 40.0, -3.0], t) == 0.0)


def test_fit_structure_matches_reference_properties(oracle):
    # tests/test_parametric.rs:32-61 and :191-205 in spirit: finite chi2,
    # per-model chi2 contains the chosen model, svi_mu length per model,
    # Laplace sigma in (0, 1e4)
    batch = synth.config_basic(2, seed=7)
    r = oracle.fit_batch(batch, fit_all_models=True, method=abi.METHOD_LAPLACE)
    assert np.all(r.model >= 0)
    for b in range(batch.n_bands):
        m = r.model[b]
        assert np.isfinite(r.pso_chi2[b])
        assert np.isfinite(r.per_model_chi2[b, m])
        assert r.per_model_chi2[b, m] == pytest.approx(r.pso_chi2[b])
        npar = abi.N_PARAMS[m]
        assert np.all(np.isfinite(r.svi_mu[b, :npar])) and np.all(np.isnan(r.svi_mu[b, npar:]))
        sig = np.exp(r.svi_log_sigma[b, :npar])
        assert np.all((sig > 0) & (sig < 1e4))
        assert r.n_obs[b] == batch.band_counts()[b]
    # each source's rank-0 band carries the MultiBazin result
    for s in range(batch.n_sources):
        bands = range(batch.source_band_offsets[s], batch.source_band_offsets[s + 1])
        r0 = [b for b in bands if r.rank[b] == 0]
        assert len(r0) == 1 and r.mb_best_k[r0[0]] >= 1


def test_fit_skips_empty_and_nonpositive_bands(oracle):
    batch = synth.config_basic(1, seed=3)
    # band 1 -> all flux negative (peak <= 0 is skipped, src/parametric.rs:3589-3592)
    o0, o1 = batch.band_obs_offsets[1], batch.band_obs_offsets[2]
    batch.flux[o0:o1] = -np.abs(batch.flux[o0:o1])
    r = oracle.fit_batch(batch, fit_all_models=True, method=abi.METHOD_LAPLACE, run_multi_bazin=False)
    assert r.model[1] == -1 and r.rank[1] == -1
    assert r.model[0] >= 0 and r.model[2] >= 0


def _two_band_villar_source(oracle):
    """The synthetic 2-band source of the reference's multiband test
    (tests/test_metal.rs:67-97): Villar [0.3, 0.01, 2.0, 10.0, 1.0, 3.0, -2.5]
    at t = 0, 1.5, ..., 43.5 in r, 0.8 x that in g, errors 5 % + 0.01."""
    t = np.arange(30) * 1.5
    r = oracle.eval_model(1, np.array([0.3, 0.01, 2.0, 10.0, 1.0, 3.0, -2.5]), t)
    g = 0.8 * r
    e = np.abs(r) * 0.05 + 0.01
    return {"ztfr": {"times": t, "values": r, "errors": e}, "ztfg": {"times": t, "values": g, "errors": e}}


def test_oracle_multiband_villar_produces_results(oracle):
    """fit_parametric with >= 2 bands and fit_all_models = false takes the
    joint multi-band Villar branch (src/parametric.rs:3750-3757): both bands
    get a Villar result with the joint (finite) cost, ranked by count
    (equal counts: input order)."""
    from lightcurve_fitting_gb300.parametric import _batch_from_sources
    batch, _ = _batch_from_sources([_two_band_villar_source(oracle)])
    r = oracle.fit_batch(batch, fit_all_models=False, method=abi.METHOD_LAPLACE, run_multi_bazin=False,
                         joint_multiband=True)
    assert list(r.model) == [1, 1] and list(r.rank) == [0, 1]
    assert np.isfinite(r.pso_chi2).all() and r.pso_chi2[0] == r.pso_chi2[1]
    assert np.array_equal(r.per_model_chi2[:, 1], r.pso_chi2)
    assert np.isnan(np.delete(r.per_model_chi2, 1, axis=1)).all()
    # each band is normalised by its own peak, so g = 0.8 r is the same
    # curve: the amplitude offset stays near its relative-prior mean
    # (-0.015 ln 10, sigma 0.08 ln 10 = 0.184)
    off = r.pso_params[1, :7] - r.pso_params[0, :7]
    assert abs(off[0] - (-0.015 * np.log(10))) < 2 * 0.08 * np.log(10)
    # without the dispatch the same source takes the per-band path
    r2 = oracle.fit_batch(batch, fit_all_models=False, method=abi.METHOD_LAPLACE, run_multi_bazin=False)
    assert np.isnan(r2.per_model_chi2[:, 1]).all() or (r2.model != 1).any()


@pytest.mark.parametrize("m", range(7))
def test_svi_step_gradient_is_the_elbo_derivative_on_detections(oracle, m):
    """The reference's SVI gradient (src/parametric.rs:2330-2393, restated)
    equals FP64 central differences of its own ELBO estimate when every
    observation is a detection (at upper limits the reference divides the
    exact pdf by the approximate CDF, so it is not the exact derivative)."""
    from lightcurve_fitting_gb300 import abi, synth
    batch = synth.config_gradient(2, seed=3)
    t, f, e = batch.bands_of(0)[0]
    band = oracle.Band(t, f, e)
    band.up = np.zeros_like(band.up)
    rng = np.random.default_rng(50 + m)
    lo, hi = [np.array(v) for v in _bounds(m)]
    npar = lo.size
    checked = 0
    for _ in range(6):
        mu = rng.uniform(lo, hi)
        mu[abi.T0_IDX[m]] = rng.uniform(t.min() - 10, t.max())
        vp = np.concatenate([mu, rng.uniform(-4.0, -1.5, npar)])
        init = mu + 0.1 * rng.standard_normal(npar)
        eps = rng.standard_normal((8, npar))
        _, g, flags = oracle.svi_elbo_grad(m, band, init, vp, eps)
        assert flags == 0
        fd = np.zeros_like(g)
        for j in range(vp.size):
            a, b = vp.copy(), vp.copy()
            a[j] += 1e-6
            b[j] -= 1e-6
            fd[j] = (oracle.svi_elbo_grad(m, band, init, a, eps)[0] - oracle.svi_elbo_grad(m, band, init, b, eps)[0]) / 2e-6
        assert np.max(np.abs(g - fd)) <= 1e-5 * max(np.max(np.abs(fd)), 1.0), (m, g, fd)
        checked += 1
    assert checked == 6


def test_svi_fit_uses_the_step_gradient(oracle):
    """One SVI step from the initial point moves mu by lr * sign(gradient)
    (Adam's first step), with the step gradient taken at the reference's own
    first Box-Muller draws (SmallRng seed 42)."""
    from lightcurve_fitting_gb300 import abi, synth
    batch = synth.config_gradient(2, seed=3)
    t, f, e = batch.bands_of(0)[0]
    band = oracle.Band(t, f, e)
    m = 0
    npar = abi.N_PARAMS[m]
    init = np.array([0.0, 0.0, float(t[np.argmax(f)]), 1.0, 3.0, -3.0])
    u = oracle.rng_f64(42, 2 * 4 * npar).reshape(4, npar, 2)
    eps = np.sqrt(-2.0 * np.log(np.maximum(u[..., 0], 1e-10))) * np.cos(2.0 * np.pi * u[..., 1])
    vp0 = np.concatenate([init, np.full(npar, -1.0)])
    _, g, _ = oracle.svi_elbo_grad(m, band, init, vp0, eps)
    mu, ls, _, steps = oracle.svi_fit(m, band, init, n_steps=1, n_samples=4)
    assert steps == 1
    moved = np.concatenate([mu, ls - np.log(4.0)]) - vp0
    # Adam's first step is lr * g / (|g| + eps) per component, toward ascent
    expect = 0.01 * g / (np.abs(g) + 1e-8)
    expect[npar:] = np.clip(vp0[npar:] + expect[npar:], -6.0, 2.0) - vp0[npar:]
    np.testing.assert_allclose(moved, expect, rtol=1e-9, atol=1e-12)


def test_golden_metzger_at_single_observations(oracle, golden):
    """The per-observation MetzgerKN of the reference's GPU kernels
    (lc_metzger_kn_at_single, cuda/models_device.h:376-456), restated in the
    oracle for the drop-in cost and SVI exports, against the reference's own
    code sampled into the golden vectors."""
    P, T, F = golden["single_m7_p"], golden["single_m7_t"], golden["single_m7_f"]
    got = np.array([[oracle.metzger_at_obs(p, t) for t in T] for p in P])
    assert np.mean(F != 0.0) > 0.5
    assert np.allclose(got, F, rtol=1e-12, atol=0.0)


def test_gpu_kernel_costs_follow_their_own_rules(oracle):
    """The reference GPU cost (cuda/models.cu:516-584) has no prior and no 1/2,
    and 1e99 for an empty source; MultiBazin with K = 1 equals Bazin's cost
    with the parameters rearranged (cuda/models.cu:295-362)."""
    from lightcurve_fitting_gb300 import synth
    batch = synth.config_basic(1, seed=4)
    t, f, e = batch.bands_of(0)[0]
    band = oracle.Band(t, f, e)
    p = np.array([0.2, 0.05, 40.0, 1.0, 3.0, -3.0])
    c = oracle.gpu_pso_cost(0, band, p)[0]
    pred = oracle.eval_model(0, p, band.t)
    tv = band.var + np.exp(p[5]) ** 2
    det = band.up == 0
    expect = np.sum((pred[det] - band.f[det]) ** 2 / tv[det] + np.log(tv[det]))
    from scipy.stats import norm
    expect -= np.sum(norm.logcdf(((band.uf - pred) / np.sqrt(tv))[~det])) if (~det).any() else 0.0
    assert abs(c - expect / band.n) <= 1e-3 * abs(expect / band.n)  # A&S erf vs scipy at the limits
    mb = np.zeros(6)
    mb[[0, 1, 2, 3, 4, 5]] = [p[0], p[2], p[3], p[4], p[1], p[5]]
    assert np.isclose(oracle.gpu_mb_cost(band, mb, 1)[0], c, rtol=1e-14)
    empty = oracle.Band.__new__(oracle.Band)
    empty.t, empty.f, empty.var, empty.uf = [np.zeros(0) for _ in range(4)]
    empty.up = np.zeros(0, np.uint8)
    assert oracle.gpu_pso_cost(0, empty, p)[0] == 1e99
    assert oracle.gpu_svi_fit(0, empty, p, p, np.ones(6), src=0)[2] == -1e99


def test_perturbation_hooks_restore_the_exact_arithmetic(oracle):
    """The oracle's test hooks (cost / gradient and swarm-position
    perturbations) move its results when set and leave them bit-identical
    once reset to 0."""
    batch = synth.config_basic(6, seed=11)
    kw = dict(fit_all_models=True, method=abi.METHOD_LAPLACE, run_multi_bazin=True)
    base = oracle.fit_batch(batch, **kw)
    moved = []
    for set_hook in (lambda: oracle.set_cost_perturbation(1e-7, 0, 1e-12),
                     lambda: oracle.set_position_perturbation(1e-13, 0)):
        set_hook()
        try:
            pert = oracle.fit_batch(batch, **kw)
        finally:
            oracle.set_cost_perturbation(0.0)
            oracle.set_position_perturbation(0.0)
        moved.append(not np.array_equal(pert.per_model_chi2, base.per_model_chi2, equal_nan=True))
    again = oracle.fit_batch(batch, **kw)
    assert all(moved)
    for f in ("model", "per_model_chi2", "pso_params", "mb_cost", "mb_per_k_cost"):
        assert np.array_equal(getattr(again, f), getattr(base, f), equal_nan=True), f


def test_oracle_on_a_ragged_batch(oracle):
    """Empty bands are skipped, one- to four-point bands and a source without
    bands are handled, MultiBazin runs on rank-0 bands of >= 5 points, and a
    source with a single band of data leaves the joint branch for the per-band
    fit (src/parametric.rs:3742-3761)."""
    import ragged
    b = ragged.batch()
    n = b.band_counts()
    for kw in (dict(fit_all_models=True, method=abi.METHOD_SVI, run_multi_bazin=True),
               dict(fit_all_models=False, method=abi.METHOD_LAPLACE, run_multi_bazin=True, joint_multiband=True)):
        r = oracle.fit_batch(b, **kw)
        assert np.array_equal(r.model >= 0, n > 0) and np.array_equal(r.n_obs, n)
        assert np.array_equal(r.mb_best_k > 0, (r.rank == 0) & (n >= 5))
    assert r.model[11] != 1 and np.all(r.model[(n > 0) & (np.arange(b.n_bands) != 11)] == 1)
