"""A ragged batch for the edge-case tests: empty bands, one- to four-point
bands, a source without bands and a source whose only non-empty band is
short, cut from the basic workload's light curves."""
import numpy as np

from lightcurve_fitting_gb300 import synth

# observations kept per band, source by source (0: an empty band)
LAYOUT = [[30, 30, 30], [30, 0, 1], [], [4, 2, 30], [0, 0, 12], [3, 30], [5, 5, 5, 5]]


def batch() -> synth.PhotometryBatch:
    base = synth.config_basic(12, seed=41)
    bands = [base.bands_of(s)[k] for s in range(base.n_sources) for k in range(3)]
    t, f, e, bo, so = [], [], [], [0], [0]
    q = 0
    for src in LAYOUT:
        for n in src:
            tt, ff, ee = bands[q]
            q += 1
            t.append(tt[:n]); f.append(ff[:n]); e.append(ee[:n])
            bo.append(bo[-1] + n)
        so.append(so[-1] + len(src))
    return synth.PhotometryBatch(np.concatenate(t), np.concatenate(f), np.concatenate(e), np.asarray(bo, np.int64),
                                 np.asarray(so, np.int32), np.zeros(len(LAYOUT), np.int32), "ragged")
