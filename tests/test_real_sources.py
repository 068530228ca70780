"""The real-source fixture and the oracle on it (CPU).

tests/golden/real_sources.npz holds the reference's 30 ZTF sources (9 classes:
SN Ia/Ib/Ic/II/IIP/IIn/IIb, cataclysmic variables, AGN, TDEs) after
build_flux_bands (src/common.rs:79-111): 83 bands of 3 to 1,005 points."""
import os
import sys

import numpy as np
import pytest

from lightcurve_fitting_gb300 import abi

import real_sources

HERE = os.path.dirname(os.path.abspath(__file__))


def test_fixture_layout():
    a = real_sources.arrays()
    bo, so = a["band_obs_offsets"], a["source_band_offsets"]
    assert so[0] == 0 and so[-1] == bo.shape[0] - 1 == a["band_names"].shape[0] == 83
    assert bo[0] == 0 and bo[-1] == a["times"].shape[0] == 15834
    assert np.all(np.diff(bo) >= 3) and np.all(np.diff(so) >= 2)
    assert a["obj_ids"].shape[0] == a["labels"].shape[0] == 30
    assert np.all(np.isfinite(a["flux"]) & (a["flux"] > 0) & np.isfinite(a["flux_err"]) & (a["flux_err"] > 0))
    for s in range(30):
        t = a["times"][bo[so[s]]:bo[so[s + 1]]]
        assert t.min() == 0.0 and np.all(np.isfinite(t))
        names = a["band_names"][so[s]:so[s + 1]]
        assert len(set(names)) == len(names) and set(names) <= {"ztfg", "ztfr", "ztfi"}


def test_fixture_is_what_the_generator_writes():
    """Regenerated from the reference's JSON where that checkout is present."""
    sys.path.insert(0, os.path.join(HERE, "golden"))
    import make_real
    if not os.path.isdir(make_real.REF):
        pytest.skip("reference checkout absent")
    fresh, saved = make_real.build(), real_sources.arrays()
    assert fresh.keys() == saved.keys()
    for k in saved:
        assert np.array_equal(fresh[k], saved[k]), k


def test_oracle_fits_every_real_band(oracle):
    """The oracle's metric path (all models, SVI, MultiBazin) on the real
    sources: every band fitted with a finite cost, ranks by descending count,
    MultiBazin on each source's rank-0 band."""
    b = real_sources.batch()
    r = oracle.fit_batch(b, fit_all_models=True, method=abi.METHOD_SVI, run_multi_bazin=True)
    assert np.all(r.model >= 0) and np.all(np.isfinite(r.pso_chi2))
    n = np.diff(b.band_obs_offsets)
    for s in range(b.n_sources):
        lo, hi = b.source_band_offsets[s], b.source_band_offsets[s + 1]
        order = sorted(range(lo, hi), key=lambda k: r.rank[k])
        assert sorted(r.rank[lo:hi]) == list(range(hi - lo))
        assert all(n[order[i]] >= n[order[i + 1]] for i in range(len(order) - 1))
        assert r.mb_best_k[order[0]] >= 1 and np.all(r.mb_best_k[order[1:]] == 0)
