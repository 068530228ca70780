"""Seeded synthetic photometry for the parametric-fit workloads.

The reference measures on synthetic Bazin light curves
(tests/synthetic.rs:54-92, tests/bench_throughput.rs) and on survey data that
is not part of its repository.  These generators produce seeded stand-ins with
the shapes, sizes and value distributions of the five workloads this project
measures:

  1. ``basic``     100 sources x 3 bands x 30 points, Bazin, t ~ U[0, 150]
  2. ``uneven``    10,000 sources x 3 bands, per-band counts
                   round(lognormal(ln 40, 0.9)) clipped to [5, 500], t ~ U[0, 300]
                   with 20 % of nights dropped, generator mix
                   {Bazin, Villar, TDE, Arnett, Magnetar}
  3. ``gradient``  4,096 sources x 3 bands x 60 points, Bazin + Villar
  4. ``precision`` 1,000 sources x 3 bands x 2,000 points, t ~ U[0, 1000],
                   A ~ LogU(10, 1e6)
  5. ``scale``     100,000 sources, counts as ``uneven`` clipped to [5, 1000]

Noise: sigma = 0.05 |F| + 5, F_obs = F + N(0, sigma^2).  Magnitudes are
derived from the noisy flux and converted back with the reference's
``build_flux_bands`` rules (src/common.rs:79-111, ZP 23.9): points with
F_obs <= 0 are dropped and times are made relative to the source's first
observation.  Output is CSR: ``times, flux, flux_err`` (float64),
``band_obs_offsets`` (int64, n_bands + 1) and ``source_band_offsets``
(int32, n_sources + 1), plus the generator id of every source.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

FACTOR = 1.0857362047581294  # 2.5 / ln 10, src/common.rs:29
ZP = 23.9

GEN_BAZIN, GEN_VILLAR, GEN_TDE, GEN_ARNETT, GEN_MAGNETAR = 0, 1, 2, 3, 4
GEN_NAMES = ["bazin", "villar", "tde", "arnett", "magnetar"]


@dataclass
class PhotometryBatch:
    """A batch of sources in the CSR layout of ``lcf_bands_csr``."""

    times: np.ndarray
    flux: np.ndarray
    flux_err: np.ndarray
    band_obs_offsets: np.ndarray
    source_band_offsets: np.ndarray
    generator: np.ndarray
    name: str = ""

    @property
    def n_sources(self) -> int:
        return int(self.source_band_offsets.shape[0] - 1)

    @property
    def n_bands(self) -> int:
        return int(self.band_obs_offsets.shape[0] - 1)

    @property
    def n_obs(self) -> int:
        return int(self.times.shape[0])

    def band_counts(self) -> np.ndarray:
        return np.diff(self.band_obs_offsets)

    def subset(self, sources) -> "PhotometryBatch":
        """Return a new batch holding the given source indices (in order)."""
        sources = np.asarray(sources, dtype=np.int64)
        t, f, e, bo, so = [], [], [], [0], [0]
        for s in sources:
            b0, b1 = self.source_band_offsets[s], self.source_band_offsets[s + 1]
            for b in range(b0, b1):
                o0, o1 = self.band_obs_offsets[b], self.band_obs_offsets[b + 1]
                t.append(self.times[o0:o1])
                f.append(self.flux[o0:o1])
                e.append(self.flux_err[o0:o1])
                bo.append(bo[-1] + (o1 - o0))
            so.append(so[-1] + (b1 - b0))
        cat = lambda xs: np.concatenate(xs) if xs else np.zeros(0)
        return PhotometryBatch(cat(t).astype(np.float64), cat(f).astype(np.float64), cat(e).astype(np.float64),
                               np.asarray(bo, np.int64), np.asarray(so, np.int32), self.generator[sources].copy(),
                               self.name)

    def bands_of(self, s: int):
        """Bands of source ``s`` as (times, flux, flux_err) tuples."""
        out = []
        for b in range(self.source_band_offsets[s], self.source_band_offsets[s + 1]):
            o0, o1 = self.band_obs_offsets[b], self.band_obs_offsets[b + 1]
            out.append((self.times[o0:o1], self.flux[o0:o1], self.flux_err[o0:o1]))
        return out


def _softplus(x):
    return np.logaddexp(0.0, x)


def _sigmoid(x):
    return 0.5 * (1.0 + np.tanh(0.5 * x))


def _light_curve(gen, t, p):
    """Noise-free flux of generator ``gen`` (per-observation arrays)."""
    A, t0, tr, tf = p["A"], p["t0"], p["tr"], p["tf"]
    ph = t - t0
    if gen == GEN_BAZIN:
        return A * np.exp(-ph / tf) * _sigmoid(ph / tr) + p["B"]
    if gen == GEN_VILLAR:
        g, beta = p["gamma"], p["beta"]
        w = _sigmoid(10.0 * (ph - g))
        right = (1.0 - beta * g) * np.exp(np.clip((g - ph) / tf, -700, 700))
        return A * _sigmoid(ph / tr) * ((1.0 - w) * (1.0 - beta * ph) + w * right)
    if gen == GEN_TDE:
        return A * _sigmoid(ph / tr) * (1.0 + _softplus(ph) / tf) ** (-p["alpha"]) + p["B"]
    if gen == GEN_ARNETT:
        ps = _softplus(ph)
        f = p["fni"]
        heat = f * np.exp(-ps / 8.8) + (1.0 - f) * np.exp(-ps / 111.3)
        return A * heat * (1.0 - np.exp(-(ps / p["tm"]) ** 2))
    # magnetar
    ps = _softplus(ph)
    return A * (1.0 + ps / p["tsd"]) ** -2 * (1.0 - np.exp(-(ps / p["tdiff"]) ** 2))


def _draw_params(rng, gen, n, amp_lo, amp_hi, t0_lo, t0_hi):
    """Per-source generator parameters (arrays of length n)."""
    p = {
        "A": np.exp(rng.uniform(np.log(amp_lo), np.log(amp_hi), n)),
        "t0": rng.uniform(t0_lo, t0_hi, n),
        "tr": rng.uniform(1.0, 15.0, n),
        "tf": rng.uniform(10.0, 80.0, n),
        "B": rng.normal(0.0, 10.0, n),
    }
    if gen == GEN_VILLAR:
        p["gamma"] = rng.uniform(1.0, 40.0, n)
        p["beta"] = rng.uniform(0.0, 0.03, n)
    elif gen == GEN_TDE:
        p["alpha"] = rng.uniform(1.0, 2.5, n)
    elif gen == GEN_ARNETT:
        m_ni = np.exp(rng.uniform(np.log(0.01), np.log(1.0), n))
        # peak luminosity scales linearly with the nickel mass (Arnett 1982)
        p["A"] = 2.0e4 * m_ni
        p["tm"] = rng.uniform(5.0, 30.0, n)
        p["fni"] = rng.uniform(0.3, 0.9, n)
    elif gen == GEN_MAGNETAR:
        b14 = np.exp(rng.uniform(np.log(0.3), np.log(30.0), n))
        p_ms = rng.uniform(1.0, 10.0, n)
        # spin-down time t_sd ~ 4.7 d B14^-2 P_ms^2 and luminosity ~ E_rot / t_sd
        # with E_rot ~ 2e52 erg P_ms^-2 (Kasen & Bildsten 2010, eqs. 1-2),
        # rescaled so the brightest sources reach 1e4 flux units.
        tsd = np.clip(4.7 * b14 ** -2 * p_ms ** 2, 0.5, 400.0)
        lum = p_ms ** -2 / tsd
        p["tsd"] = tsd
        p["A"] = np.clip(1.0e4 * lum / lum.max(), 100.0, 1.0e4)
        p["tdiff"] = rng.uniform(10.0, 40.0, n)
    return p


def generate(n_sources: int, counts, gens, *, seed: int, t_span: float, drop_nights: float,
             amp_lo: float = 100.0, amp_hi: float = 1.0e4, t0_range=(30.0, 80.0), name: str = "") -> PhotometryBatch:
    """Generic generator.  ``counts`` is (n_sources, 3) points per band before
    the F_obs <= 0 drop; ``gens`` is the generator id of each source."""
    rng = np.random.default_rng(seed)
    counts = np.asarray(counts, dtype=np.int64)
    gens = np.asarray(gens, dtype=np.int64)
    n_bands = 3 * n_sources
    band_n = counts.reshape(-1)
    total = int(band_n.sum())
    band_of_obs = np.repeat(np.arange(n_bands), band_n)
    src_of_obs = band_of_obs // 3
    # observation times: uniform within kept nights
    if drop_nights > 0.0:
        n_nights = int(np.ceil(t_span))
        keep = rng.random(n_nights) >= drop_nights
        kept = np.flatnonzero(keep).astype(np.float64)
        if kept.size == 0:
            kept = np.arange(n_nights, dtype=np.float64)
        nights = kept[rng.integers(0, kept.size, total)]
        t = np.minimum(nights + rng.random(total), t_span)
    else:
        t = rng.uniform(0.0, t_span, total)
    # sort times within each band
    order = np.lexsort((t, band_of_obs))
    t = t[order]
    # per-source parameters, by generator
    flux = np.empty(total)
    band_scale = rng.uniform(0.6, 1.4, n_bands)
    for g in np.unique(gens):
        srcs = np.flatnonzero(gens == g)
        p = _draw_params(rng, int(g), srcs.size, amp_lo, amp_hi, *t0_range)
        sel = np.isin(src_of_obs, srcs)
        idx = np.searchsorted(srcs, src_of_obs[sel])
        pp = {k: v[idx] for k, v in p.items()}
        pp["A"] = pp["A"] * band_scale[band_of_obs[sel]]
        flux[sel] = _light_curve(int(g), t[sel], pp)
    sigma = 0.05 * np.abs(flux) + 5.0
    f_obs = flux + rng.normal(0.0, 1.0, total) * sigma
    keep_obs = f_obs > 0.0
    # mag round trip of build_flux_bands (src/common.rs:32-36, 79-111)
    with np.errstate(divide="ignore", invalid="ignore"):
        mag = ZP - 2.5 * np.log10(np.where(keep_obs, f_obs, 1.0))
        mag_err = FACTOR * sigma / np.where(keep_obs, f_obs, 1.0)
    fl = 10.0 ** (-0.4 * (mag - ZP))
    fe = mag_err / FACTOR * fl
    keep_obs &= np.isfinite(fl) & np.isfinite(fe) & (fl > 0) & (fe > 0)
    t, fl, fe, band_of_obs = t[keep_obs], fl[keep_obs], fe[keep_obs], band_of_obs[keep_obs]
    band_counts = np.bincount(band_of_obs, minlength=n_bands)
    bo = np.zeros(n_bands + 1, np.int64)
    np.cumsum(band_counts, out=bo[1:])
    # times relative to each source's first observation
    src = band_of_obs // 3
    tmin = np.full(n_sources, np.inf)
    np.minimum.at(tmin, src, t)
    tmin[~np.isfinite(tmin)] = 0.0
    t = t - tmin[src]
    so = (np.arange(n_sources + 1) * 3).astype(np.int32)
    return PhotometryBatch(t.astype(np.float64), fl.astype(np.float64), fe.astype(np.float64), bo, so,
                           gens.astype(np.int32), name)


def uneven_counts(rng, n_sources, lo, hi):
    return np.clip(np.round(rng.lognormal(np.log(40.0), 0.9, (n_sources, 3))), lo, hi).astype(np.int64)


def config_basic(n_sources: int = 100, seed: int = 1) -> PhotometryBatch:
    counts = np.full((n_sources, 3), 30)
    return generate(n_sources, counts, np.zeros(n_sources, np.int64), seed=seed, t_span=150.0,
                    drop_nights=0.0, name="basic-100x3x30")


def config_uneven(n_sources: int = 10_000, seed: int = 2, max_count: int = 500) -> PhotometryBatch:
    rng = np.random.default_rng(seed + 1000)
    counts = uneven_counts(rng, n_sources, 5, max_count)
    gens = rng.integers(0, 5, n_sources)
    return generate(n_sources, counts, gens, seed=seed, t_span=300.0, drop_nights=0.2,
                    name=f"uneven-{n_sources}x3-lognormal40")


def config_gradient(n_sources: int = 4096, seed: int = 3) -> PhotometryBatch:
    rng = np.random.default_rng(seed + 1000)
    gens = rng.integers(0, 2, n_sources)
    return generate(n_sources, np.full((n_sources, 3), 60), gens, seed=seed, t_span=150.0,
                    drop_nights=0.0, name="gradient-4096x3x60")


def config_precision(n_sources: int = 1000, seed: int = 4) -> PhotometryBatch:
    return generate(n_sources, np.full((n_sources, 3), 2000), np.zeros(n_sources, np.int64), seed=seed,
                    t_span=1000.0, drop_nights=0.0, amp_lo=10.0, amp_hi=1.0e6, name="precision-1000x3x2000")


def config_scale(n_sources: int = 100_000, seed: int = 5) -> PhotometryBatch:
    rng = np.random.default_rng(seed + 1000)
    counts = uneven_counts(rng, n_sources, 5, 1000)
    gens = rng.integers(0, 5, n_sources)
    return generate(n_sources, counts, gens, seed=seed, t_span=300.0, drop_nights=0.2,
                    name=f"scale-{n_sources}x3")


CONFIGS = {
    "basic": config_basic,
    "uneven": config_uneven,
    "gradient": config_gradient,
    "precision": config_precision,
    "scale": config_scale,
}
