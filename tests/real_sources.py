"""The reference's 30 real ZTF sources (tests/fixtures/real_sources.json,
the input of its tests/test_real_data.rs) as a PhotometryBatch, loaded from
tests/golden/real_sources.npz (written by tests/golden/make_real.py)."""
import os

import numpy as np

from lightcurve_fitting_gb300 import synth

PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "real_sources.npz")


def arrays() -> dict:
    with np.load(PATH) as z:
        return {k: z[k] for k in z.files}


def batch() -> synth.PhotometryBatch:
    a = arrays()
    n = a["source_band_offsets"].shape[0] - 1
    return synth.PhotometryBatch(a["times"], a["flux"], a["flux_err"], a["band_obs_offsets"],
                                 a["source_band_offsets"], np.zeros(n, np.int32), "real_ztf_30")
