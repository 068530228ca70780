"""Generate tests/golden/real_sources.npz from the reference's real-data
fixture, tests/fixtures/real_sources.json: 30 ZTF sources (object id, class
label, per-band times, magnitudes and magnitude errors), the input of the
reference's own tests/test_real_data.rs.

Each source's magnitudes go through build_flux_bands (src/common.rs:79-111,
the Python mirror parametric.build_flux_bands: times relative to the source's
earliest time, mag -> flux with zero point 23.9, non-finite or non-positive
points dropped), and the batch is stored in the library's CSR layout: times,
flux, flux_err (FP64), band_obs_offsets (int64), source_band_offsets (int32),
plus the band names and object ids.

Run from the repository root:  python tests/golden/make_real.py
(LCF_REFERENCE_DIR, default /root/reference, is the reference checkout.)
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from lightcurve_fitting_gb300 import parametric  # noqa: E402

REF = os.environ.get("LCF_REFERENCE_DIR", "/root/reference")


def build(ref_dir: str = REF) -> dict:
    """The fixture's arrays, from the reference's real_sources.json."""
    with open(os.path.join(ref_dir, "tests", "fixtures", "real_sources.json")) as fh:
        fixtures = json.load(fh)
    sources, ids, labels = [], [], []
    for src in fixtures:
        t, m, e, b = [], [], [], []
        for name, bv in src["bands"].items():
            t += list(bv["times"])
            m += list(bv["values"])
            e += list(bv["errors"])
            b += [name] * len(bv["times"])
        sources.append(parametric.build_flux_bands(t, m, e, b))
        ids.append(src["obj_id"])
        labels.append(src.get("label_name", ""))
    batch, names = parametric._batch_from_sources(sources)
    return dict(times=batch.times, flux=batch.flux, flux_err=batch.flux_err,
                band_obs_offsets=batch.band_obs_offsets, source_band_offsets=batch.source_band_offsets,
                band_names=np.array([n for ns in names for n in ns]), obj_ids=np.array(ids),
                labels=np.array(labels))


def main() -> None:
    arrays = build()
    np.savez_compressed(os.path.join(HERE, "real_sources.npz"), **arrays)
    n = np.diff(arrays["band_obs_offsets"])
    print(f"{len(arrays['obj_ids'])} sources, {n.size} bands, {n.sum()} observations (per band {n.min()}..{n.max()})")


if __name__ == "__main__":
    main()
