"""Parity criteria stated against the oracle's own sensitivity, shared by the
GPU tests of the fit: the oracle refitted under rounding-sized perturbations
of its costs and gradients (oracle.set_cost_perturbation), and the model-
selection check that counts a disagreement with the oracle as explained only
when it is a near tie (BIC gap below 1e-3 of the best), a band where a
perturbed oracle changes its choice or one of the two polished costs, or a
band where the GPU's polish of one of the two models ended on another local
optimum."""
import numpy as np

from lightcurve_fitting_gb300 import abi


# (cost, salt, gradient) relative perturbations of the oracle
PERTURBATIONS = [(1e-7, 0, 0.0), (1e-7, 1, 0.0), (1e-9, 2, 0.0), (0.0, 3, 1e-12), (0.0, 4, 1e-14)]


def perturbed(oracle, batch, rel, salt=0, grad_rel=0.0, **kw):
    oracle.set_cost_perturbation(rel, salt, grad_rel)
    try:
        return oracle.fit_batch(batch, **kw)
    finally:
        oracle.set_cost_perturbation(0.0)


def _bic(r, b, m):
    n = r.n_obs[b]
    return 2.0 * r.per_model_chi2[b, m] * n + abi.N_PARAMS[m] * np.log(n)


def _tie(r, b, m1, m2):
    gap = abs(_bic(r, b, m1) - _bic(r, b, m2))
    return gap <= 1e-3 * abs(_bic(r, b, m2)) + 1e-9


def _moved(pr, ref, b, m):
    return abs(pr.per_model_chi2[b, m] - ref.per_model_chi2[b, m]) > 1e-4 * max(abs(ref.per_model_chi2[b, m]), 1e-12)


def selection_check(res, ref, perts):
    """(agreement, floor, bad, n, n_orc): floor = min(0.99, the lowest
    agreement of a perturbed oracle with the oracle); bad lists the
    disagreements that are neither near ties, nor at bands where a perturbed
    oracle moves, nor at bands where the GPU's polish of one of the two models
    ended elsewhere; n counts the disagreements that are not near ties, n_orc
    the most such disagreements of a perturbed oracle with the oracle."""
    fitted = ref.model >= 0
    assert np.array_equal(res.model >= 0, fitted)
    assert np.array_equal(res.rank, ref.rank)
    agree = res.model[fitted] == ref.model[fitted]
    bad, n = [], 0
    for b in np.flatnonzero(fitted)[~agree]:
        mg, mo = int(res.model[b]), int(ref.model[b])
        if _tie(ref, b, mg, mo):
            continue
        n += 1
        unstable = any(pr.model[b] != mo or _moved(pr, ref, b, mg) or _moved(pr, ref, b, mo) for pr in perts)
        elsewhere = _moved(res, ref, b, mg) or _moved(res, ref, b, mo)
        if not (unstable or elsewhere):
            bad.append((int(b), mo, mg))
    n_orc = max(int(sum(1 for b in np.flatnonzero(fitted) if pr.model[b] != ref.model[b]
                        and not _tie(ref, b, int(pr.model[b]), int(ref.model[b])))) for pr in perts)
    floor = min([0.99] + [float(np.mean(pr.model[fitted] == ref.model[fitted])) for pr in perts])
    return float(agree.mean()), floor, bad, n, n_orc


def within(a, b, tol):
    return np.abs(a - b) <= tol * np.maximum(np.abs(b), 1e-12)


# The joint multi-band Villar fit (fit_parametric_multiband).  Its 200-particle,
# 1500-iteration swarm follows the reference's trajectory in double-float but
# compares FP32 costs, which lie within 5e-7 of the FP64 joint cost (median
# 5e-8 - 9e-8, measured on the real and synthetic sources); the reference's
# own search moves under cost perturbations of 1e-6 on 15-70 % of sources,
# by up to 100 %.  So the search is held to the oracle perturbed at 1e-6.
JOINT_PERTURBATIONS = [(1e-6, 0, 0.0), (1e-6, 1, 0.0)]


def joint_vector(res, batch, s):
    """The joint parameter vector of source s (reference band, then the
    offsets of the other bands in rank order) and its fitted bands."""
    bands = range(batch.source_band_offsets[s], batch.source_band_offsets[s + 1])
    fitted = sorted([b for b in bands if res.rank[b] >= 0], key=lambda b: res.rank[b])
    ref = res.pso_params[fitted[0], :7]
    return np.concatenate([ref] + [res.pso_params[b, :7] - ref for b in fitted[1:]]), fitted


def joint_search_rel(res, ref, batch):
    """Per source: (joint cost of res - of ref) / max(|of ref|, 1)."""
    out = []
    for s in range(batch.n_sources):
        _, fitted = joint_vector(ref, batch, s)
        a, b = res.pso_chi2[fitted[0]], ref.pso_chi2[fitted[0]]
        out.append((a - b) / max(abs(b), 1.0))
    return np.array(out)


def check_joint(g, oracle, batch, kw):
    """The joint fit g against the oracle: dispatch and outputs, the reported
    cost against the FP64 joint cost at g's own vector (1e-6), and the search
    (median departure 1e-6; no more sources departing by 1e-4 than the oracle
    perturbed at 1e-6 has)."""
    r = oracle.fit_batch(batch, **kw)
    assert np.array_equal(g.rank, r.rank) and np.array_equal(g.model, r.model)
    assert set(g.model[g.model >= 0]) == {1}
    fitted_all = g.model >= 0
    assert np.array_equal(g.per_model_chi2[fitted_all, 1], g.pso_chi2[fitted_all])
    assert np.isnan(np.delete(g.per_model_chi2[fitted_all], 1, axis=1)).all()
    rel_fn = []
    for s in range(batch.n_sources):
        p, fitted = joint_vector(g, batch, s)
        c_gpu = g.pso_chi2[fitted[0]]
        assert all(g.pso_chi2[b] == c_gpu for b in fitted)
        c_fp64 = oracle.joint_cost(batch, s, p)
        rel_fn.append(abs(c_gpu - c_fp64) / max(abs(c_fp64), 1.0))
    assert max(rel_fn) < 1e-6, rel_fn
    rel = joint_search_rel(g, r, batch)
    n_gpu = int(np.sum(np.abs(rel) > 1e-4))
    n_orc = max(int(np.sum(np.abs(joint_search_rel(perturbed(oracle, batch, *p, **kw), r, batch)) > 1e-4))
                for p in JOINT_PERTURBATIONS)
    assert np.median(np.abs(rel)) < 1e-6 and n_gpu <= n_orc, (np.median(np.abs(rel)), n_gpu, n_orc, rel)
