"""The parity criteria of the GPU tests (criteria.py), checked on the CPU with
the oracle alone: they accept a result the reference itself could give (the
oracle under a rounding-sized perturbation stands in for the GPU) and reject
planted mistakes (wrong models, a wrong joint cost), so that a GPU test passes
only on the reference's own behaviour."""
import copy

import numpy as np
import pytest

from lightcurve_fitting_gb300 import abi, synth

from criteria import PERTURBATIONS, _moved, _tie, check_joint, perturbed, selection_check

KW = dict(fit_all_models=True, method=abi.METHOD_LAPLACE, run_multi_bazin=False)


@pytest.fixture(scope="module")
def fits(oracle):
    batch = synth.config_uneven(40, seed=17)
    ref = oracle.fit_batch(batch, **KW)
    perts = [perturbed(oracle, batch, *p, **KW) for p in PERTURBATIONS]
    stand_in = perturbed(oracle, batch, 1e-9, 9, **KW)
    return batch, ref, perts, stand_in


def test_selection_check_accepts_the_reference_under_rounding(fits):
    _, ref, perts, stand_in = fits
    frac, floor, bad, n, n_orc = selection_check(stand_in, ref, perts)
    assert frac >= floor and not bad and n <= max(n_orc, 1), (frac, floor, bad, n, n_orc)


def test_selection_check_rejects_planted_wrong_models(fits):
    """Bands whose choice is stable under every perturbation get another
    model that is no near tie and whose cost no perturbation moves: each one
    is reported."""
    _, ref, perts, _ = fits
    wrong = copy.deepcopy(ref)
    planted = []
    for b in np.flatnonzero(ref.model >= 0):
        if len(planted) == 4:
            break
        mo = int(ref.model[b])
        if any(p.model[b] != mo or _moved(p, ref, b, mo) for p in perts):
            continue
        for m in range(8):
            if m == mo or not np.isfinite(ref.per_model_chi2[b, m]) or _tie(ref, b, m, mo):
                continue
            if any(_moved(p, ref, b, m) for p in perts):
                continue
            wrong.model[b] = m
            planted.append(int(b))
            break
    assert len(planted) == 4
    frac, floor, bad, n, n_orc = selection_check(wrong, ref, perts)
    assert {b for b, _, _ in bad} == set(planted)


def test_check_joint_rejects_a_wrong_cost(oracle):
    """The joint check on the oracle's own joint fit (perturbed at 1e-9 as the
    stand-in) passes; with one source's reported cost moved by 1e-5 it fails."""
    batch = synth.config_basic(6, seed=23)
    kw = dict(fit_all_models=False, method=abi.METHOD_LAPLACE, run_multi_bazin=False, joint_multiband=True)
    g = perturbed(oracle, batch, 1e-9, 7, **kw)
    check_joint(g, oracle, batch, kw)
    bad = copy.deepcopy(g)
    s = 2
    lo, hi = batch.source_band_offsets[s], batch.source_band_offsets[s + 1]
    bad.pso_chi2[lo:hi] *= 1.0 + 1e-5
    with pytest.raises(AssertionError):
        check_joint(bad, oracle, batch, kw)
